"""Serving with continuous batching (ptgpu_server_*): a request's pixels and
colours equal a single-scene context's draw_frame(spp) from the same seed
streams, whether the request runs alone or among others that arrive while it
is on the GPU, and whatever the step quantum; scenes are evicted under LRU
when the budget is small and rebuilt on their next request."""
import threading

import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

FLAGS = abi.FLAG_TREELET | abi.treelet_sweeps(2)


def _scenes():
    return [scenes.icosphere_scene(level=4, seed=3),
            scenes.icosphere_scene(level=5, seed=4, n_tris=6000),
            scenes.cornell_spheres(),
            scenes.icosphere_scene(level=6, seed=5, n_tris=30000)]


def _reference(sh, lc, cam, w, h, spp, seed):
    import ptgpu_pc_gb300 as pt
    with pt.Context(w, h, accel=abi.ACCEL_BVH) as ctx:
        ctx.set_shapes(sh, lc)
        ctx.build(abi.ACCEL_BVH, FLAGS)
        ctx.set_camera(cam)
        ctx.set_seeds(pt.make_seeds(seed, 2 * w * h))
        px = ctx.draw_frame(spp)
        col = ctx.get_colors().view(np.float32).reshape(-1, 3).copy()
    return px, col


REQS = [(0, 48, 32, 5, 11), (1, 40, 40, 9, 12), (2, 32, 24, 3, 13), (3, 64, 48, 6, 14),
        (0, 24, 24, 2, 15), (2, 16, 16, 12, 16)]


@pytest.mark.parametrize("quantum,flags", [(1, 0), (4, 0), (4, abi.SERVER_ALL_ACTIVE)])
def test_served_results_equal_single_contexts_alone_and_mixed(quantum, flags, built_lib):
    import ptgpu_pc_gb300 as pt
    sc = _scenes()
    with pt.Server(budget_bytes=8 << 30, quantum=quantum, flags=flags) as srv:
        ids = [srv.add_scene(sh, lc, FLAGS) for sh, lc, _ in sc]
        # alone: one request at a time
        alone = []
        for s, w, h, spp, seed in REQS:
            t = srv.submit(ids[s], sc[s][2], w, h, spp, seed)
            alone.append(srv.wait(t))
        # mixed: all at once, from two threads, waited in reverse order
        tickets = [None] * len(REQS)

        def submit(part):
            for i in part:
                s, w, h, spp, seed = REQS[i]
                tickets[i] = srv.submit(ids[s], sc[s][2], w, h, spp, seed)

        th = [threading.Thread(target=submit, args=(range(k, len(REQS), 2),)) for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        mixed = [None] * len(REQS)
        for i in reversed(range(len(REQS))):
            mixed[i] = srv.wait(tickets[i])
        info = srv.info()
    assert info["requests_done"] == 2 * len(REQS)
    assert info["builds"] == len(sc)            # each scene built once, then resident
    assert any(m[2]["steps"] > 1 for m in mixed) or quantum > 8
    for i, (s, w, h, spp, seed) in enumerate(REQS):
        px, col = _reference(sc[s][0], sc[s][1], sc[s][2], w, h, spp, seed)
        for got in (alone[i], mixed[i]):
            assert np.array_equal(got[1].view(np.uint32), col.view(np.uint32)), "request %d" % i
            assert np.array_equal(got[0], px), "request %d pixels" % i


def test_lru_eviction_under_a_small_budget(built_lib):
    import ptgpu_pc_gb300 as pt
    sc = _scenes()
    # room for the largest scene's slots and little more
    with pt.Server(budget_bytes=7 << 20, quantum=4) as srv:
        ids = [srv.add_scene(sh, lc, FLAGS) for sh, lc, _ in sc]
        order = [3, 1, 3, 0, 1, 2, 3]
        outs = []
        for s in order:
            t = srv.submit(ids[s], sc[s][2], 32, 32, 3, 100 + s)
            outs.append(srv.wait(t))
        info = srv.info()
    assert info["evictions"] > 0
    assert info["builds"] > len(set(order))
    for s, got in zip(order, outs):
        px, col = _reference(sc[s][0], sc[s][1], sc[s][2], 32, 32, 3, 100 + s)
        assert np.array_equal(got[1].view(np.uint32), col.view(np.uint32))


def test_request_beyond_the_budget_is_rejected(built_lib):
    import ptgpu_pc_gb300 as pt
    sh, lc, cam = scenes.icosphere_scene(level=4, seed=3)
    with pt.Server(budget_bytes=1 << 20, quantum=4) as srv:
        sid = srv.add_scene(sh, lc)
        t = srv.submit(sid, cam, 512, 512, 1, 1)
        with pytest.raises(pt.PtgpuError) as e:
            srv.wait(t)
        assert e.value.status == abi.E_RANGE
        with pytest.raises(pt.PtgpuError) as e:
            srv.submit(99, cam, 8, 8, 1, 1)
        assert e.value.status == abi.E_INVAL


def test_fill_cap_runs_a_gpu_filling_request_alone(built_lib):
    """The default step policy: a request whose pixels fill the GPU by itself
    (1536^2, over 15 pixels per resident lane) takes its steps alone, so the
    small requests that arrive behind it wait and then share their own steps:
    6 + 12 steps at quantum 1 (the largest small request has 12 passes).
    Every result still equals the single-scene context's."""
    import ptgpu_pc_gb300 as pt
    sc = _scenes()
    big = (0, 1536, 1536, 6, 21)
    with pt.Server(budget_bytes=8 << 30, quantum=1) as srv:
        ids = [srv.add_scene(sh, lc, FLAGS) for sh, lc, _ in sc]
        reqs = [big] + REQS
        tickets = [srv.submit(ids[s], sc[s][2], w, h, spp, seed) for s, w, h, spp, seed in reqs]
        outs = [srv.wait(t) for t in tickets]
        info = srv.info()
    assert outs[0][2]["steps"] == big[3]
    assert info["steps"] == big[3] + max(r[3] for r in REQS)
    for (s, w, h, spp, seed), got in zip(reqs, outs):
        px, col = _reference(sc[s][0], sc[s][1], sc[s][2], w, h, spp, seed)
        assert np.array_equal(got[1].view(np.uint32), col.view(np.uint32)), (w, h, spp)
        assert np.array_equal(got[0], px), (w, h, spp)
