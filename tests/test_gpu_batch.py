"""Batched scenes (ptgpu_batch_*): each scene's BVH arrays, colours and pixels
must equal what a single-scene context produces from the same shapes, camera,
seeds, passes and build flags -- byte for byte, since the batch runs the same
arithmetic in a shared index space."""
import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _scene_set():
    out = []
    sh, lc, cam = scenes.icosphere_scene(level=3, seed=5)
    out.append((sh, lc, cam, 64, 48, 3))
    sh, lc, cam = scenes.icosphere_scene(level=5, seed=7, n_tris=3000)
    out.append((sh, lc, cam, 40, 40, 2))
    sh, lc, cam = scenes.cornell_spheres()
    out.append((sh, lc, cam, 32, 24, 4))
    sh, lc, cam = scenes.icosphere_scene(level=6, seed=9, n_tris=20000)
    out.append((sh, lc, cam, 24, 32, 1))
    # tiny trees: 2 shapes (no treelet round applies) and 3
    near = scenes.camera([0.5, 0.5, 3.0])
    out.append((scenes.triangle_soup(2, seed=31), 0, near, 16, 16, 2))
    out.append((scenes.triangle_soup(3, seed=32), 0, near, 16, 8, 3))
    return out


def _single(sh, lc, cam, w, h, passes, seeds, build_flags, ctx_flags, frames):
    import ptgpu_pc_gb300 as pt
    res = []
    with pt.Context(w, h, accel=abi.ACCEL_BVH, flags=ctx_flags) as ctx:
        ctx.set_shapes(sh, lc)
        ctx.build(abi.ACCEL_BVH, build_flags)
        btn, btl = ctx.get_bvh()
        ctx.set_camera(cam)
        ctx.set_seeds(seeds)
        for _ in range(frames):
            px = ctx.draw_frame(passes).copy()
            res.append((px, ctx.get_colors().view(np.float32).reshape(-1, 3).copy()))
    return btn, btl, res


@pytest.mark.parametrize("build_flags,ctx_flags", [
    (0, 0),
    (abi.FLAG_TREELET | abi.treelet_sweeps(2), 0),
    (0, abi.FLAG_ARGS_RTL),
])
def test_batch_matches_single_scene_contexts(build_flags, ctx_flags, built_lib):
    import ptgpu_pc_gb300 as pt
    sset = _scene_set()
    seeds = [pt.make_seeds(100 + i, 2 * w * h) for i, (_, _, _, w, h, _) in enumerate(sset)]
    with pt.Batch(flags=ctx_flags) as b:
        ids = [b.add(sh, lc, cam, w, h, p, sd) for (sh, lc, cam, w, h, p), sd in zip(sset, seeds)]
        b.build(build_flags)
        frames = []
        for _ in range(2):
            b.render()
            frames.append([(b.pixels(i), b.colors(i)) for i in ids])
        bvhs = [b.bvh(i) for i in ids]
        info = b.info()
    assert info["shapes"] == sum(len(s[0]) for s in sset)
    assert info["samples"] == sum(w * h * p for (_, _, _, w, h, p) in sset)
    for k, ((sh, lc, cam, w, h, p), sd) in enumerate(zip(sset, seeds)):
        btn, btl, res = _single(sh, lc, cam, w, h, p, sd, build_flags, ctx_flags, 2)
        assert bvhs[k][0].tobytes() == btn.tobytes(), "scene %d btn" % k
        assert bvhs[k][1].tobytes() == btl.tobytes(), "scene %d btl" % k
        for f in range(2):
            assert np.array_equal(frames[f][k][1].view(np.uint32), res[f][1].view(np.uint32)), \
                "scene %d frame %d colours" % (k, f)
            assert np.array_equal(frames[f][k][0], res[f][0]), "scene %d frame %d pixels" % (k, f)


def test_batch_tune_keeps_results(built_lib):
    import ptgpu_pc_gb300 as pt
    sset = _scene_set()[:3]
    seeds = [pt.make_seeds(7 + i, 2 * w * h) for i, (_, _, _, w, h, _) in enumerate(sset)]

    def run(tune):
        with pt.Batch() as b:
            ids = [b.add(sh, lc, cam, w, h, p, sd) for (sh, lc, cam, w, h, p), sd in zip(sset, seeds)]
            b.build(abi.FLAG_TREELET)
            if tune:
                b.tune()
            b.render()
            info = b.info()
            return [b.colors(i) for i in ids], info

    a, _ = run(False)
    c, info = run(True)
    assert info["block"] in (64, 96, 128) and info["refill"] in (16, 20, 24)
    assert info["stack"] in (32, 64, 128) and info["tree_depth"] > 0
    for x, y in zip(a, c):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_batch_errors(built_lib):
    import ptgpu_pc_gb300 as pt
    sh, lc, cam = scenes.icosphere_scene(level=2)
    with pt.Batch() as b:
        with pytest.raises(pt.PtgpuError) as e:
            b.render()
        assert e.value.status == abi.E_STATE
        with pytest.raises(pt.PtgpuError) as e:
            b.add(sh[:1], 0, cam, 8, 8, 1, pt.make_seeds(1, 128))
        assert e.value.status == abi.E_INVAL
        with pytest.raises(pt.PtgpuError) as e:
            b.build()
        assert e.value.status == abi.E_STATE
