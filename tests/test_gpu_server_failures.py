"""Serving failure paths, all injected on the host: a cancelled pending
request, a cancelled active request, a scene file that disappears before
its scene is rebuilt after an LRU eviction, and the progressive preview of a
running request.  After each, the server keeps serving, later results are
right, and the slot counts show nothing leaked.  (The reference has no
request notion: these paths have no counterpart there.)"""
import os
import time

import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _context_frame(sh, lc, cam, w, h, spp, seed, flags=0):
    import ptgpu_pc_gb300 as pt
    with pt.Context(w, h, accel=abi.ACCEL_BVH) as ctx:
        ctx.set_shapes(sh, lc)
        ctx.build(abi.ACCEL_BVH, flags)
        ctx.set_camera(cam)
        ctx.set_seeds(pt.make_seeds(seed, 2 * w * h))
        px = ctx.draw_frame(spp)
        return px, ctx.get_colors().view(np.float32).reshape(-1, 3).copy()


def _wait_until(pred, timeout=60.0):
    t0 = time.time()
    while not pred():
        if time.time() - t0 > timeout:
            raise AssertionError("condition not reached in %.0f s" % timeout)
        time.sleep(0.002)


def _passes(srv, ticket):
    """Passes a request's preview holds (0 while it waits for admission)."""
    import ptgpu_pc_gb300 as pt
    try:
        return srv.preview(ticket, want_pixels=False, want_colors=False)[2]
    except pt.PtgpuError as e:
        if e.status == abi.E_STATE:
            return 0
        raise


def test_cancel_pending_and_active_requests(built_lib):
    import ptgpu_pc_gb300 as pt
    sh, lc, cam = scenes.icosphere_scene(level=4, seed=3)
    # pixels of one 512x512 request fit the budget, two do not: the second
    # waits in the queue while the first runs
    with pt.Server(budget_bytes=10 << 20, quantum=1) as srv:
        sid = srv.add_scene(sh, lc)
        t_long = srv.submit(sid, cam, 512, 512, 4000, 21)   # one pass per step: seconds
        t_pend = srv.submit(sid, cam, 512, 512, 2, 22)
        _wait_until(lambda: srv.info()["active_requests"] == 1)
        assert srv.info()["pending_requests"] == 1
        srv.cancel(t_pend)                                  # pending: leaves the queue
        with pytest.raises(pt.PtgpuError) as e:
            srv.wait(t_pend)
        assert e.value.status == abi.E_CANCELED
        # the running one: cancelled after it has rendered a few steps
        _wait_until(lambda: _passes(srv, t_long) >= 2)
        srv.cancel(t_long)
        with pytest.raises(pt.PtgpuError) as e:
            srv.wait(t_long)
        assert e.value.status == abi.E_CANCELED
        info = srv.info()
        assert info["pixel_slots_used"] == 0 and info["active_requests"] == 0
        # the server keeps serving, with the same results as a context
        t = srv.submit(sid, cam, 48, 40, 3, 23)
        px, col, _ = srv.wait(t)
    rpx, rcol = _context_frame(sh, lc, cam, 48, 40, 3, 23)
    assert np.array_equal(px, rpx) and np.array_equal(col.view(np.uint32), rcol.view(np.uint32))


def test_progressive_preview_equals_partial_frame(built_lib):
    """A preview of a running request holds exactly the passes it reports:
    its colours equal a context's frame of that many passes."""
    import ptgpu_pc_gb300 as pt
    sh, lc, cam = scenes.icosphere_scene(level=5, seed=4, n_tris=8000)
    w, h, spp, seed = 256, 256, 48, 31
    with pt.Server(budget_bytes=1 << 30, quantum=1) as srv:
        sid = srv.add_scene(sh, lc)
        t = srv.submit(sid, cam, w, h, spp, seed)
        _wait_until(lambda: _passes(srv, t) >= 1)
        ppx, pcol, passes = srv.preview(t)
        px, col, st = srv.wait(t)
        # after the request finished and before wait() the preview is the final image
    assert 1 <= passes <= spp
    rpx, rcol = _context_frame(sh, lc, cam, w, h, passes, seed)
    assert np.array_equal(pcol.view(np.uint32), rcol.view(np.uint32))
    assert np.array_equal(ppx, rpx)
    fpx, fcol = _context_frame(sh, lc, cam, w, h, spp, seed)
    assert np.array_equal(col.view(np.uint32), fcol.view(np.uint32))


def test_preview_before_admission_is_a_state_error(built_lib):
    import ptgpu_pc_gb300 as pt
    sh, lc, cam = scenes.icosphere_scene(level=3, seed=5)
    with pt.Server(budget_bytes=10 << 20, quantum=1) as srv:
        sid = srv.add_scene(sh, lc)
        t1 = srv.submit(sid, cam, 512, 512, 4000, 41)
        t2 = srv.submit(sid, cam, 512, 512, 1, 42)         # waits for t1's pixels
        _wait_until(lambda: srv.info()["active_requests"] == 1)
        with pytest.raises(pt.PtgpuError) as e:
            srv.preview(t2)
        assert e.value.status == abi.E_STATE
        srv.cancel(t1)
        with pytest.raises(pt.PtgpuError):
            srv.wait(t1)
        srv.wait(t2, want_pixels=False, want_colors=False)


def test_scene_file_gone_before_rebuild(built_lib, tmp_path):
    """A served file scene is evicted, its file deleted, and requested again:
    the rebuild fails with E_IO, its slots go back to the arenas, and the
    other scenes keep being served."""
    import ptgpu_pc_gb300 as pt
    path = scenes.write_model_scene(str(tmp_path), 20000, seed=6)
    other, olc, ocam = scenes.icosphere_scene(level=6, seed=7, n_tris=30000)
    with pt.Context(8, 8) as ctx:
        ctx.read_scene(path)
        fcam = ctx.get_camera()
    # room for one of the two scenes' shape slots at a time
    with pt.Server(budget_bytes=8 << 20, quantum=4) as srv:
        fid = srv.add_scene_file(path)
        oid = srv.add_scene(other, olc)
        srv.wait(srv.submit(fid, fcam, 32, 32, 2, 51), want_pixels=False, want_colors=False)
        srv.wait(srv.submit(oid, ocam, 32, 32, 2, 52), want_pixels=False, want_colors=False)
        info = srv.info()
        assert info["evictions"] >= 1 and info["resident_scenes"] == 1
        before = info["shape_slots_used"]
        os.remove(path)
        t = srv.submit(fid, fcam, 32, 32, 2, 53)
        with pytest.raises(pt.PtgpuError) as e:
            srv.wait(t)
        assert e.value.status == abi.E_IO
        info = srv.info()
        assert info["shape_slots_used"] <= before          # the failed build kept nothing
        assert info["pixel_slots_used"] == 0
        px, col, _ = srv.wait(srv.submit(oid, ocam, 40, 32, 3, 54))
    rpx, rcol = _context_frame(other, olc, ocam, 40, 32, 3, 54)
    assert np.array_equal(col.view(np.uint32), rcol.view(np.uint32))
