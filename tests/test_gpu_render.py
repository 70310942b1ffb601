"""Path tracer (RadianceGPU, rendering_kernel.cl:1072-1150) vs the oracle on
the same seed streams: relative RMSE of the float accumulation buffer below
1e-3 and mean luminance within 3 sigma (sigma from seed replicas), for the
no-accel, BVH and KD-tree modes."""
import os

import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

RMSE_TOL = 1e-3


def _oracle_cam(cam, w, h, orc):
    c = np.array(cam, abi.CAMERA)
    c["width"], c["height"] = w, h
    return orc.update_camera(c)


def _gpu_render(shapes, lc, cam, w, h, seeds, passes, accel, max_depth=0, flags=0, chunks=None):
    import ptgpu_pc_gb300 as pt
    with pt.Context(w, h, accel=accel, max_depth=max_depth, flags=flags) as ctx:
        ctx.set_shapes(shapes, lc)
        ctx.build(accel)
        ctx.set_camera(cam)
        ctx.set_seeds(seeds)
        for p in (chunks or [passes]):
            pix = ctx.draw_frame(p)
        col = ctx.get_colors()
        sd = ctx.get_seeds()
    return col, pix, sd


def _oracle_render(shapes, lc, cam, w, h, seeds, passes, accel, orc, max_depth=6, rtl=False,
                   portable_trig=True):
    if accel == abi.ACCEL_BVH:
        _, btn, btl, _ = orc.build_bvh(shapes)
        acc = orc.make_accel(accel, btn, btl)
    elif accel == abi.ACCEL_KDTREE:
        acc = orc.make_accel(accel, kd=orc.KD(shapes))
    else:
        acc = orc.make_accel(accel)
    return orc.render(shapes, lc, _oracle_cam(cam, w, h, orc), w, h, seeds, passes, accel=acc,
                      max_depth=max_depth, arg_order_rtl=rtl, portable_trig=portable_trig)


def _rel_rmse(a, b):
    a = a.view(np.float32).reshape(-1, 3).astype(np.float64)
    b = b.view(np.float32).reshape(-1, 3).astype(np.float64)
    return np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-30)


@pytest.mark.parametrize("accel", [abi.ACCEL_NONE, abi.ACCEL_BVH, abi.ACCEL_KDTREE])
def test_render_cornell_spheres(accel, built_lib, orc):
    shapes, lc, cam = scenes.cornell_spheres()
    w = h = 64
    seeds = orc.make_seeds(1, 2 * w * h)
    g_col, g_pix, g_sd = _gpu_render(shapes, lc, cam, w, h, seeds, 4, accel)
    o_col, o_pix, o_sd = _oracle_render(shapes, lc, cam, w, h, seeds, 4, accel, orc)
    assert _rel_rmse(g_col, o_col) < RMSE_TOL
    same = (g_col.view(np.uint8).reshape(-1, 12) == o_col.view(np.uint8).reshape(-1, 12)).all(1)
    assert same.mean() > 0.999
    # pixels: the gamma pack uses each platform's powf; channels within 1
    d = np.abs(g_pix.view(np.uint8).astype(int) - o_pix.view(np.uint8).astype(int))
    assert d.max() <= 1


@pytest.mark.parametrize("accel", [abi.ACCEL_BVH, abi.ACCEL_KDTREE])
def test_render_icosphere(accel, built_lib, orc):
    shapes, lc, cam = scenes.icosphere_scene(level=4)
    w = h = 48
    seeds = orc.make_seeds(2, 2 * w * h)
    g_col, g_pix, g_sd = _gpu_render(shapes, lc, cam, w, h, seeds, 2, accel, max_depth=8)
    o_col, o_pix, o_sd = _oracle_render(shapes, lc, cam, w, h, seeds, 2, accel, orc, max_depth=8)
    assert _rel_rmse(g_col, o_col) < RMSE_TOL
    assert (g_sd == o_sd).mean() > 0.98


def test_render_arg_order_rtl(built_lib, orc):
    """With PTGPU_FLAG_ARGS_RTL the GPU follows the order the reference
    source gets from g++ (the oracle is pinned to that build)."""
    shapes, lc, cam = scenes.icosphere_scene(level=3)
    w = h = 32
    seeds = orc.make_seeds(3, 2 * w * h)
    g_col, _, _ = _gpu_render(shapes, lc, cam, w, h, seeds, 2, abi.ACCEL_BVH,
                              flags=abi.FLAG_ARGS_RTL)
    o_col, _, _ = _oracle_render(shapes, lc, cam, w, h, seeds, 2, abi.ACCEL_BVH, orc, rtl=True)
    assert _rel_rmse(g_col, o_col) < RMSE_TOL


def test_progressive_equals_single_call(built_lib, orc):
    """4 passes in one DrawFrame == 1+3 passes (the running mean continues)."""
    shapes, lc, cam = scenes.icosphere_scene(level=3)
    w = h = 32
    seeds = orc.make_seeds(4, 2 * w * h)
    a = _gpu_render(shapes, lc, cam, w, h, seeds, 4, abi.ACCEL_BVH)
    b = _gpu_render(shapes, lc, cam, w, h, seeds, 4, abi.ACCEL_BVH, chunks=[1, 3])
    assert a[0].tobytes() == b[0].tobytes()
    assert (a[1] == b[1]).all() and (a[2] == b[2]).all()


def test_handout_order_keeps_results(built_lib, orc):
    """Frames after the first hand pixels out in decreasing work of the frame
    before; results do not depend on the order: 1+1+1+1 passes in four calls
    (three of them reordered) == 4 passes in one call (row order)."""
    shapes, lc, cam = scenes.icosphere_scene(level=4)
    w, h = 160, 120
    seeds = orc.make_seeds(5, 2 * w * h)
    a = _gpu_render(shapes, lc, cam, w, h, seeds, 4, abi.ACCEL_BVH)
    b = _gpu_render(shapes, lc, cam, w, h, seeds, 4, abi.ACCEL_BVH, chunks=[1, 1, 1, 1])
    assert a[0].tobytes() == b[0].tobytes()
    assert (a[1] == b[1]).all() and (a[2] == b[2]).all()


def test_render_obj_model_fixture(built_lib, orc):
    """The reference's own OBJ scene, loaded by the reference loader when the
    golden fixture was made, rendered in all three modes."""
    path = os.path.join(os.path.dirname(__file__), "golden", "obj_model_scene.npz")
    z = np.load(path)
    shapes = z["shapes"].view(abi.SHAPE).reshape(-1)
    lc = int(z["light_cnt"])
    cam = z["camera"].view(abi.CAMERA)[0]
    w, h = 40, 30
    seeds = orc.make_seeds(5, 2 * w * h)
    for accel in (abi.ACCEL_NONE, abi.ACCEL_BVH, abi.ACCEL_KDTREE):
        g_col, _, _ = _gpu_render(shapes, lc, cam, w, h, seeds, 2, accel)
        o_col, _, _ = _oracle_render(shapes, lc, cam, w, h, seeds, 2, accel, orc)
        assert _rel_rmse(g_col, o_col) < RMSE_TOL, accel


def test_mean_luminance_within_3_sigma(built_lib, orc):
    """Mean radiance of the GPU image within 3 sigma of the oracle's, sigma
    from 8 independent seed replicas of the oracle."""
    shapes, lc, cam = scenes.icosphere_scene(level=3)
    w = h = 24
    means = []
    for r in range(8):
        seeds = orc.make_seeds(100 + r, 2 * w * h)
        o_col, _, _ = _oracle_render(shapes, lc, cam, w, h, seeds, 2, abi.ACCEL_BVH, orc)
        means.append(o_col.view(np.float32).mean())
    sigma = np.std(means, ddof=1)
    seeds = orc.make_seeds(100, 2 * w * h)
    g_col, _, _ = _gpu_render(shapes, lc, cam, w, h, seeds, 2, abi.ACCEL_BVH)
    assert abs(g_col.view(np.float32).mean() - means[0]) <= 3 * sigma


@pytest.mark.parametrize("accel", [abi.ACCEL_NONE, abi.ACCEL_BVH, abi.ACCEL_KDTREE])
def test_wavefront_matches_lane_tracer(accel, built_lib, orc):
    """The wavefront kernels and the per-lane tracer compute the same image,
    bit for bit, including progressive calls that continue the running mean."""
    shapes, lc, cam = scenes.icosphere_scene(level=3)
    if accel == abi.ACCEL_NONE:
        shapes, lc, cam = scenes.cornell_spheres()
    w, h = 40, 36
    seeds = orc.make_seeds(6, 2 * w * h)
    a = _gpu_render(shapes, lc, cam, w, h, seeds, 3, accel, max_depth=7, chunks=[2, 1])
    b = _gpu_render(shapes, lc, cam, w, h, seeds, 3, accel, max_depth=7, chunks=[2, 1],
                    flags=abi.FLAG_WAVEFRONT)
    assert a[0].tobytes() == b[0].tobytes()
    assert (a[1] == b[1]).all() and (a[2] == b[2]).all()


def test_wavefront_vs_oracle(built_lib, orc):
    shapes, lc, cam = scenes.icosphere_scene(level=4)
    w = h = 48
    seeds = orc.make_seeds(7, 2 * w * h)
    g_col, _, g_sd = _gpu_render(shapes, lc, cam, w, h, seeds, 2, abi.ACCEL_BVH, max_depth=8,
                                 flags=abi.FLAG_WAVEFRONT)
    o_col, _, o_sd = _oracle_render(shapes, lc, cam, w, h, seeds, 2, abi.ACCEL_BVH, orc, max_depth=8)
    assert _rel_rmse(g_col, o_col) < RMSE_TOL
    assert (g_sd == o_sd).mean() > 0.99
