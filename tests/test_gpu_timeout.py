"""The radix sort's bounded look-back wait (the decoupled look-back of each
onesweep pass) giving up, without any GPU fault: with the context's wait
limit at 0 every sort tile after the first gives up at its first wait, the
build returns PTGPU_E_TIMEOUT (the reference has no bounded wait: its host
sort never waits, and its OpenCL errors are only logged, CLBVH.cpp:12-20),
and the same context then builds the oracle's tree with the default limit."""
import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def test_lookback_timeout_then_context_still_builds(built_lib, orc):
    import ptgpu_pc_gb300 as pt
    shapes = scenes.triangle_soup(200_000, seed=51)     # 40 sort tiles
    _, o_btn, o_btl, _ = orc.build_bvh(shapes)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, 0)
        ctx.set_wait_limit(0)
        with pytest.raises(pt.PtgpuError) as ei:
            ctx.build(abi.ACCEL_BVH)
        assert ei.value.status == abi.E_TIMEOUT
        assert b"look-back" in pt.lib().ptgpu_last_error()
        # rendering needs a built structure: the failed build left none
        with pytest.raises(pt.PtgpuError):
            ctx.trace_closest(scenes.random_rays(16, seed=52))
        ctx.set_wait_limit(abi.WAIT_LIMIT_DEFAULT)
        ctx.build(abi.ACCEL_BVH)
        btn, btl = ctx.get_bvh()
        assert btl.tobytes() == o_btl.tobytes()
        assert btn.tobytes() == o_btn.tobytes()
        rays = scenes.random_rays(10_000, seed=53)
        t, ids, hit = ctx.trace_closest(rays)
    ot, oid, ohit = orc.trace_closest(shapes, rays, orc.make_accel(abi.ACCEL_BVH, o_btn, o_btl, fast=True))
    assert np.array_equal(hit, ohit)


def test_single_tile_build_never_waits(built_lib, orc):
    """A build of one sort tile (at most 5,120 shapes) has no look-back, so
    even a zero wait limit succeeds."""
    import ptgpu_pc_gb300 as pt
    shapes = scenes.triangle_soup(5000, seed=54)
    _, o_btn, o_btl, _ = orc.build_bvh(shapes)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, 0)
        ctx.set_wait_limit(0)
        ctx.build(abi.ACCEL_BVH)
        btn, btl = ctx.get_bvh()
    assert btn.tobytes() == o_btn.tobytes() and btl.tobytes() == o_btl.tobytes()
