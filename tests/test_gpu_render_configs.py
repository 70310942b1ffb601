"""Render parity at the benchmark configurations (RadianceGPU,
rendering_kernel.cl:1072-1150), against the oracle in the mode pinned to the
reference compiled here: sin/cos from libm and the two random arguments of a
light sample drawn right to left, the order g++ gives the reference source
(the GPU runs with PTGPU_FLAG_ARGS_RTL).  Both sides consume the same
per-pixel seed streams.

  config 1: Cornell box of 9 spheres, 256x256, 16 spp, depth 6, no
            acceleration, the whole frame;
  config 2: displaced level-6 icosphere + walls + area light (81,934
            shapes), 512x512, 16 spp, depth 8, BVH and KD tree; the oracle
            renders every 32nd row (16 rows x 512 pixels: pixels are
            independent, so those rows of the GPU frame are an exact
            sub-image).

Tolerances: relative RMSE of the float accumulation buffer below 1e-3 and
the mean radiance within 3 sigma of the oracle's, sigma taken from 8 seed
replicas of the oracle at the same configuration.  The GPU's own sine and
cosine differ from libm's in the last bit for some arguments, so bit
identity is asserted against the oracle run with those functions
(portable_trig=True) and only reported against the libm mode.

Config 1's light is a r=600 sphere whose cap pokes 0.27 below the ceiling;
nearly all light samples are blocked and the image is made of rare samples
that see the cap, with near-singular 1/len^2 weights (8 seed replicas give
frame means from 0.39 to 1.07).  A last-bit change of one bounce direction
moves such a sample by orders of magnitude: the oracle itself, run once with
libm and once with the GPU's sine and cosine, differs by a relative RMSE of
0.22 on 0.7 % of the pixels.  For config 1 the libm comparison therefore
asserts the mean within 3 sigma and the identical-pixel fraction, and the
1e-3 RMSE is asserted against the portable mode (where it holds with almost
every pixel bit-identical)."""
import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

RMSE_TOL = 1e-3
REPLICAS = 8


def _cam(cam, w, h, orc):
    c = np.array(cam, abi.CAMERA)
    c["width"], c["height"] = w, h
    return orc.update_camera(c)


def _gpu(shapes, lc, cam, w, h, seeds, passes, accel, max_depth):
    import ptgpu_pc_gb300 as pt
    with pt.Context(w, h, accel=accel, max_depth=max_depth, flags=abi.FLAG_ARGS_RTL) as ctx:
        ctx.set_shapes(shapes, lc)
        ctx.build(accel)
        ctx.set_camera(cam)
        ctx.set_seeds(seeds)
        pix = ctx.draw_frame(passes)
        return ctx.get_colors(), pix, ctx.get_seeds()


def _f(col, idx=None):
    a = col.view(np.float32).reshape(-1, 3)
    return a if idx is None else a[idx]


def _rel_rmse(a, b):
    a = a.astype(np.float64); b = b.astype(np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-30))


def _identical(a, b):
    return float((a.view(np.uint32).reshape(len(a), -1) == b.view(np.uint32).reshape(len(b), -1)).all(1).mean())


# ---------------------------------------------------------------------------
# config 1: the whole frame
# ---------------------------------------------------------------------------
C1 = dict(w=256, h=256, spp=16, depth=6)


@pytest.fixture(scope="module")
def config1(orc):
    shapes, lc, cam = scenes.cornell_spheres()
    w, h = C1["w"], C1["h"]
    ocam = _cam(cam, w, h, orc)
    acc = orc.make_accel(abi.ACCEL_NONE)
    out = {"shapes": shapes, "lc": lc, "cam": cam, "seeds": orc.make_seeds(1, 2 * w * h)}
    means = []
    for r in range(REPLICAS):
        seeds = orc.make_seeds(1 + r, 2 * w * h)
        col, _, sd = orc.render(shapes, lc, ocam, w, h, seeds, C1["spp"], accel=acc,
                                max_depth=C1["depth"], arg_order_rtl=True)
        means.append(float(_f(col).mean()))
        if r == 0:
            out["libm"] = (col, sd)
    out["means"] = means
    col, _, sd = orc.render(shapes, lc, ocam, w, h, out["seeds"], C1["spp"], accel=acc,
                            max_depth=C1["depth"], arg_order_rtl=True, portable_trig=True)
    out["portable"] = (col, sd)
    return out


def test_config1_cornell_spheres_full_frame(config1, built_lib, parity_report):
    c = config1
    g_col, g_pix, g_sd = _gpu(c["shapes"], c["lc"], c["cam"], C1["w"], C1["h"], c["seeds"],
                              C1["spp"], abi.ACCEL_NONE, C1["depth"])
    g = _f(g_col)
    p_col, p_sd = c["portable"]
    l_col, l_sd = c["libm"]
    rel_pt, same_pt = _rel_rmse(g, _f(p_col)), _identical(g, _f(p_col))
    rel_lm, same_lm = _rel_rmse(g, _f(l_col)), _identical(g, _f(l_col))
    sigma = float(np.std(c["means"], ddof=1))
    parity_report("config1_cornell_spheres_256x256_16spp", rel_rmse_portable=rel_pt,
                  identical_portable=same_pt, rel_rmse_libm=rel_lm, identical_libm=same_lm,
                  mean_gpu=float(g.mean()), mean_oracle_libm=c["means"][0], sigma_replicas=sigma,
                  seeds_equal_portable=float((g_sd == p_sd).mean()))
    assert rel_pt < RMSE_TOL
    assert same_pt > 0.999
    assert (g_sd == p_sd).mean() > 0.999
    assert abs(float(g.mean()) - c["means"][0]) <= 3 * sigma
    assert same_lm > 0.98


# ---------------------------------------------------------------------------
# config 2: every 32nd row of the frame, BVH and KD tree
# ---------------------------------------------------------------------------
C2 = dict(w=512, h=512, spp=16, depth=8)
ROWS = list(range(16, 512, 32))


def _rows_render(orc, shapes, lc, ocam, seeds, acc, portable=False):
    w, h = C2["w"], C2["h"]
    seeds = np.array(seeds, np.uint32, copy=True)
    colors = np.zeros(w * h, abi.VEC)
    for y in ROWS:
        colors, _, seeds = orc.render(shapes, lc, ocam, w, h, seeds, C2["spp"], accel=acc,
                                      max_depth=C2["depth"], arg_order_rtl=True, rows=(y, y + 1),
                                      colors=colors, portable_trig=portable)
    return colors, seeds


def _row_index():
    w, h = C2["w"], C2["h"]
    # colors are stored row-flipped (RadianceGPU writes (H - y - 1) * W + x)
    col_idx = np.concatenate([np.arange((h - y - 1) * w, (h - y) * w) for y in ROWS])
    seed_idx = np.concatenate([np.arange(2 * y * w, 2 * (y + 1) * w) for y in ROWS])
    return col_idx, seed_idx


@pytest.fixture(scope="module")
def config2(orc):
    shapes, lc, cam = scenes.icosphere_scene(level=6)
    w, h = C2["w"], C2["h"]
    ocam = _cam(cam, w, h, orc)
    _, btn, btl, _ = orc.build_bvh(shapes)
    accs = {abi.ACCEL_BVH: orc.make_accel(abi.ACCEL_BVH, btn, btl, fast=True),
            abi.ACCEL_KDTREE: orc.make_accel(abi.ACCEL_KDTREE, kd=orc.KD(shapes), fast=True)}
    col_idx, _ = _row_index()
    means = []
    for r in range(REPLICAS):
        col, _ = _rows_render(orc, shapes, lc, ocam, orc.make_seeds(1 + r, 2 * w * h),
                              accs[abi.ACCEL_BVH])
        means.append(float(_f(col, col_idx).mean()))
    return {"shapes": shapes, "lc": lc, "cam": cam, "ocam": ocam, "accs": accs,
            "seeds": orc.make_seeds(1, 2 * w * h), "means": means}


@pytest.mark.parametrize("accel", [abi.ACCEL_BVH, abi.ACCEL_KDTREE])
def test_config2_icosphere_rows(accel, config2, built_lib, orc, parity_report):
    c = config2
    col_idx, seed_idx = _row_index()
    g_col, g_pix, g_sd = _gpu(c["shapes"], c["lc"], c["cam"], C2["w"], C2["h"], c["seeds"],
                              C2["spp"], accel, C2["depth"])
    g = _f(g_col, col_idx)
    l_col, l_sd = _rows_render(orc, c["shapes"], c["lc"], c["ocam"], c["seeds"], c["accs"][accel])
    p_col, p_sd = _rows_render(orc, c["shapes"], c["lc"], c["ocam"], c["seeds"], c["accs"][accel],
                               portable=True)
    l, p = _f(l_col, col_idx), _f(p_col, col_idx)
    rel_lm, same_lm = _rel_rmse(g, l), _identical(g, l)
    rel_pt, same_pt = _rel_rmse(g, p), _identical(g, p)
    sigma = float(np.std(c["means"], ddof=1))
    parity_report("config2_icosphere81934_512x512_16spp_%s" % ("bvh" if accel == abi.ACCEL_BVH else "kd"),
                  rows=len(ROWS), rel_rmse_libm=rel_lm, identical_libm=same_lm,
                  rel_rmse_portable=rel_pt, identical_portable=same_pt,
                  mean_gpu=float(g.mean()), mean_oracle_libm=float(l.mean()), sigma_replicas=sigma,
                  seeds_equal_libm=float((g_sd[seed_idx] == l_sd[seed_idx]).mean()))
    assert rel_lm < RMSE_TOL
    assert abs(float(g.mean()) - float(l.mean())) <= 3 * sigma
    assert rel_pt < RMSE_TOL
    assert same_pt > 0.999
    assert (g_sd[seed_idx] == p_sd[seed_idx]).mean() > 0.999


# ---------------------------------------------------------------------------
# config 1 with the opt-in throughput Russian roulette (rr_depth = 3)
# ---------------------------------------------------------------------------
def test_config1_russian_roulette_option(config1, built_lib, orc, parity_report):
    """Config 1's "Russian roulette after depth 3": ptgpu_config.rr_depth = 3
    on the GPU and the same roulette in the oracle consume the same randoms
    and give the same image (portable sine/cosine: bit for bit); the
    reference itself has no such roulette, so rr_depth = 0 stays the
    default."""
    import ptgpu_pc_gb300 as pt
    c = config1
    w, h = C1["w"], C1["h"]
    with pt.Context(w, h, accel=abi.ACCEL_NONE, max_depth=C1["depth"], flags=abi.FLAG_ARGS_RTL,
                    rr_depth=3) as ctx:
        ctx.set_shapes(c["shapes"], c["lc"])
        ctx.build(abi.ACCEL_NONE)
        ctx.set_camera(c["cam"])
        ctx.set_seeds(c["seeds"])
        ctx.draw_frame(C1["spp"])
        g_col, g_sd = ctx.get_colors(), ctx.get_seeds()
    ocam = _cam(c["cam"], w, h, orc)
    o_col, _, o_sd = orc.render(c["shapes"], c["lc"], ocam, w, h, c["seeds"], C1["spp"],
                                accel=orc.make_accel(abi.ACCEL_NONE), max_depth=C1["depth"],
                                arg_order_rtl=True, portable_trig=True, rr_depth=3)
    g, o = _f(g_col), _f(o_col)
    parity_report("config1_rr_depth3", rel_rmse_portable=_rel_rmse(g, o), identical_portable=_identical(g, o),
                  seeds_equal=float((g_sd == o_sd).mean()),
                  seeds_changed_vs_plain=float((g_sd != c["portable"][1]).mean()))
    assert _rel_rmse(g, o) < RMSE_TOL
    assert _identical(g, o) > 0.999
    assert (g_sd == o_sd).mean() > 0.999
    # the roulette draws randoms: the seed streams move on past the plain ones
    assert (g_sd != c["portable"][1]).mean() > 0.5


def test_russian_roulette_rejected_with_wavefront(built_lib):
    import ptgpu_pc_gb300 as pt
    with pytest.raises(pt.PtgpuError):
        pt.Context(16, 16, flags=abi.FLAG_WAVEFRONT, rr_depth=3)
