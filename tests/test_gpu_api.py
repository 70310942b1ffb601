"""C-ABI behaviour on the GPU: status codes, call order, round trips."""
import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def test_draw_before_build_is_state_error(built_lib):
    import ptgpu_pc_gb300 as pt
    with pt.Context(16, 16) as ctx:
        ctx.set_shapes(scenes.cornell_spheres()[0], 1)
        with pytest.raises(pt.PtgpuError) as e:
            ctx.draw_frame(1)
        assert e.value.status == abi.E_STATE


def test_missing_scene_is_io_error(built_lib):
    import ptgpu_pc_gb300 as pt
    with pt.Context(16, 16) as ctx:
        with pytest.raises(pt.PtgpuError) as e:
            ctx.read_scene("/nonexistent/scene.txt")
        assert e.value.status == abi.E_IO


def test_seed_roundtrip_and_bvh_install(built_lib, orc):
    import ptgpu_pc_gb300 as pt
    shapes, lc, cam = scenes.icosphere_scene(level=2)
    _, btn, btl, _ = orc.build_bvh(shapes)
    with pt.Context(16, 16) as ctx:
        ctx.set_shapes(shapes, lc)
        s = pt.make_seeds(9, 2 * 16 * 16)
        ctx.set_seeds(s)
        assert (ctx.get_seeds() == s).all()
        ctx.set_bvh(btn, btl)           # the ReInit upload of caller-built trees
        ctx.set_camera(cam)
        ctx.draw_frame(1)
        g_btn, g_btl = ctx.get_bvh()
        assert g_btn.tobytes() == btn.tobytes() and g_btl.tobytes() == btl.tobytes()


def test_kdtree_export_and_range(built_lib, orc):
    import ptgpu_pc_gb300 as pt
    small = scenes.triangle_soup(500, seed=2)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(small, 0)
        ctx.build(abi.ACCEL_KDTREE)
        kng, kn = ctx.get_kdtree()
    okng, okn, st = orc.KD(small).heap()
    assert st == 0 and kng.tobytes() == okng.tobytes() and (kn == okn).all()
    big, lc, _ = scenes.icosphere_scene(level=6)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(big, lc)
        ctx.build(abi.ACCEL_KDTREE)
        with pytest.raises(pt.PtgpuError) as e:
            ctx.get_kdtree()
        assert e.value.status == abi.E_RANGE


def test_trace_device_pointers(built_lib, orc):
    torch = pytest.importorskip("torch")
    import ptgpu_pc_gb300 as pt
    shapes = scenes.triangle_soup(10_000, seed=3)
    rays = scenes.random_rays(4096, seed=3)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, 0)
        ctx.build(abi.ACCEL_BVH)
        ref = ctx.trace_closest(rays)
        d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
        d_t = torch.zeros(len(rays), dtype=torch.float32, device="cuda")
        d_id = torch.zeros(len(rays), dtype=torch.int32, device="cuda")
        d_hit = torch.zeros(len(rays), dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        ctx.trace_closest_device(d_rays.data_ptr(), len(rays), d_t.data_ptr(), d_id.data_ptr(),
                                 d_hit.data_ptr())
        ctx.synchronize()
        assert np.array_equal(d_t.cpu().numpy(), ref[0])
        assert np.array_equal(d_id.cpu().numpy().view(np.uint32), ref[1])
