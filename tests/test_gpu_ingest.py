"""Scene ingestion without a host copy of the shapes (ptgpu_stream_scene,
ptgpu_server_add_scene_file) against ptgpu_read_scene on the same file: the
same shapes byte for byte, the same light records (checked through renders),
the same BVH, KD tree and pixels; served file scenes equal served shape
arrays, also after eviction forces them to be read again."""
import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _load(path, stream, w=48, h=32):
    import ptgpu_pc_gb300 as pt
    ctx = pt.Context(w, h, accel=abi.ACCEL_BVH)
    wl = ctx.stream_scene(path) if stream else ctx.read_scene(path)
    return ctx, wl


@pytest.fixture(scope="module")
def scene_file(tmp_path_factory):
    return scenes.write_model_scene(tmp_path_factory.mktemp("ingest"), 40_000, seed=5)


def test_stream_scene_equals_read_scene(scene_file, built_lib):
    import ptgpu_pc_gb300 as pt
    outs = []
    for stream in (False, True):
        ctx, wl = _load(scene_file, stream)
        with ctx:
            n, lc = ctx.shape_count()
            shapes = ctx.get_shapes()                 # before any build: the loader's records
            cam = ctx.get_camera()
            ctx.build(abi.ACCEL_BVH)
            btn, btl = ctx.get_bvh()
            shapes_b = ctx.get_shapes()               # after the build: index / morton / bound
            ctx.set_seeds(pt.make_seeds(9, 2 * ctx.width * ctx.height))
            px = ctx.draw_frame(4)
            col = ctx.get_colors().view(np.uint32).copy()
        outs.append((wl, n, lc, shapes, cam, btn, btl, shapes_b, px, col))
    a, b = outs
    assert a[0] == b[0] and a[1] == b[1] and a[2] == b[2]
    assert a[2] > 1000                                # the emitting model's triangles are lights
    assert a[3].tobytes() == b[3].tobytes()
    assert a[4].tobytes() == b[4].tobytes()
    assert a[5].tobytes() == b[5].tobytes() and a[6].tobytes() == b[6].tobytes()
    assert a[7].tobytes() == b[7].tobytes()
    assert np.array_equal(a[8], b[8]) and np.array_equal(a[9], b[9])


def test_stream_scene_kd_paths(scene_file, built_lib):
    """After streaming, the host KD build (which needs host shapes) and the
    GPU one give read_scene's trees, and get_shapes keeps the KD numbering."""
    res = []
    for stream in (False, True):
        ctx, _ = _load(scene_file, stream)
        with ctx:
            rays = scenes.random_rays(20_000, seed=6)
            rays["o"] = rays["o"] * 40.0 - 20.0
            per = []
            for flags in (abi.FLAG_KD_HOST, 0):
                ctx.build(abi.ACCEL_KDTREE, flags)
                t, i, hit = ctx.trace_closest(rays)
                per.append((t.view(np.uint32).copy(), i.copy(), hit.copy()))
            shapes = ctx.get_shapes()
        res.append((per, shapes))
    for (ta, ia, ha), (tb, ib, hb) in zip(res[0][0], res[1][0]):
        assert ha.sum() > 0
        assert np.array_equal(ha, hb) and np.array_equal(ta, tb) and np.array_equal(ia, ib)
    assert res[0][1].tobytes() == res[1][1].tobytes()


def test_stream_scene_large_model(tmp_path, built_lib):
    path = scenes.write_model_scene(tmp_path, 600_000, seed=7)
    got = []
    for stream in (False, True):
        ctx, _ = _load(path, stream, 8, 8)
        with ctx:
            got.append((ctx.shape_count(), ctx.get_shapes()))
    assert got[0][0] == got[1][0]
    assert got[0][1].tobytes() == got[1][1].tobytes()


def test_served_scene_file_equals_shape_array(scene_file, tmp_path, built_lib):
    """A served scene given by its file renders like the same shapes given as
    an array; with a budget that holds one scene at a time the file scene is
    evicted and read again from the file, with the same result."""
    import ptgpu_pc_gb300 as pt
    ctx, _ = _load(scene_file, False, 8, 8)
    with ctx:
        shapes = ctx.get_shapes()
        lc = ctx.shape_count()[1]
        cam = ctx.get_camera()
    other = scenes.write_model_scene(tmp_path, 30_000, seed=8)
    flags = abi.FLAG_TREELET | abi.treelet_sweeps(2)
    w, h, spp = 32, 24, 3
    with pt.Server(budget_bytes=64 << 30, quantum=2) as srv:
        a = srv.add_scene(shapes, lc, flags)
        b = srv.add_scene_file(scene_file, flags)
        ra = srv.wait(srv.submit(a, cam, w, h, spp, 21))
        rb = srv.wait(srv.submit(b, cam, w, h, spp, 21))
    assert np.array_equal(ra[0], rb[0])
    assert np.array_equal(ra[1].view(np.uint32), rb[1].view(np.uint32))
    # small budget: two file scenes alternate, each rebuilt from its file
    with pt.Server(budget_bytes=12 << 20, quantum=2) as srv:
        b = srv.add_scene_file(scene_file, flags)
        c = srv.add_scene_file(other, flags)
        outs = [srv.wait(srv.submit(s, cam, w, h, spp, 21)) for s in (b, c, b)]
        info = srv.info()
    assert info["evictions"] >= 2 and info["builds"] >= 3
    assert np.array_equal(outs[2][0], ra[0])
    assert np.array_equal(outs[2][1].view(np.uint32), ra[1].view(np.uint32))
