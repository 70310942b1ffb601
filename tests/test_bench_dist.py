"""The benchmark's multi-rank plumbing on CPU: two gloo ranks, launched the
way torchrun sets them up (RANK / WORLD_SIZE / MASTER_* in the environment).
Each rank renders its own replica, so the only cross-rank steps are the
barriers and the max over ranks of the timed seconds."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    try:
        os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                           "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
        sys.path.insert(0, ROOT)
        import bench
        r, w, local, pg = bench.dist_setup(world)
        assert (r, w, local) == (rank, world, rank) and pg is not None
        bench.barrier(pg)
        # rank r "timed" 1.5 + r seconds: every rank reports the slowest
        slowest = bench.reduce_max(1.5 + r, pg, "cpu")
        bench.barrier(pg)
        pg.destroy_process_group()
        q.put((rank, slowest))
    except Exception as e:  # reported to the parent
        q.put((rank, repr(e)))


def test_two_gloo_ranks_take_the_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 2.5, 1: 2.5}


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        assert k not in os.environ or os.environ[k] in ("0", "1")
    r, w, local, pg = bench.dist_setup(1)
    assert pg is None
    assert bench.reduce_max(3.25, pg, "cpu") == 3.25


def test_reference_arm_other_ranks_exit_without_work():
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup, gpus, ref_seconds = 1, 0, 2, 1.0

    # rank 1 of 2 returns before loading the scene or the oracle
    assert bench.run_reference(Args(), 1, 2, None) is None
