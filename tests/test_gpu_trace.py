"""Closest-hit queries (Intersect, rendering_kernel.cl:194-363) vs the oracle:
primitive id bit-exact except rays whose hit lies within 1e-6 (barycentric)
of a triangle edge, t within 1e-5 relative."""
import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu

T_RTOL = 1e-5
EDGE = 1e-6


def _barycentric_margin(shapes, ids, rays, t):
    """min(u, v, 1-u-v) of each hit in float64 (edge exclusion)."""
    s = shapes[ids]
    p1, p2, p3 = (s[f].astype(np.float64) for f in ("p1", "p2", "p3"))
    o = rays["o"].astype(np.float64)
    d = rays["d"].astype(np.float64)
    x = o + t[:, None].astype(np.float64) * d
    e1, e2, ep = p2 - p1, p3 - p1, x - p1
    d11 = (e1 * e1).sum(1); d12 = (e1 * e2).sum(1); d22 = (e2 * e2).sum(1)
    dp1 = (ep * e1).sum(1); dp2 = (ep * e2).sum(1)
    den = d11 * d22 - d12 * d12
    den[den == 0] = 1
    v = (d22 * dp1 - d12 * dp2) / den
    w = (d11 * dp2 - d12 * dp1) / den
    m = np.minimum(np.minimum(v, w), 1 - v - w)
    m[s["type"] != abi.TRIANGLE] = 1.0
    return m


def _check(shapes, rays, g, o):
    gt, gid, ghit = g
    ot, oid, ohit = o
    both = (ghit == 1) & (ohit == 1) & (gt < 1e20) & (ot < 1e20)
    only = (ghit != ohit)
    # disagreement on hit/miss only for grazing cases
    assert only.mean() < 1e-4, "hit/miss disagree on %d rays" % only.sum()
    rel = np.abs(gt[both] - ot[both]) / np.maximum(np.abs(ot[both]), 1e-30)
    assert (rel <= T_RTOL).mean() > 0.9999, "t differs: max rel %g" % rel.max()
    diff = both & (gid != oid)
    if diff.any():
        m_o = _barycentric_margin(shapes, oid[diff], rays[diff], ot[diff])
        m_g = _barycentric_margin(shapes, gid[diff], rays[diff], gt[diff])
        assert ((m_o < EDGE) | (m_g < EDGE) | (np.abs(gt[diff] - ot[diff]) == 0)).all(), \
            "%d id mismatches away from edges" % diff.sum()
    return both.sum(), diff.sum()


def test_closest_bvh_soup(built_lib, orc):
    import ptgpu_pc_gb300 as pt
    shapes = scenes.triangle_soup(200_000, seed=8)
    rays = scenes.random_rays(50_000, seed=9)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, 0)
        ctx.build(abi.ACCEL_BVH)
        g = ctx.trace_closest(rays)
        btn, btl = ctx.get_bvh()
    acc = orc.make_accel(abi.ACCEL_BVH, btn, btl)
    o = orc.trace_closest(shapes, rays, acc)
    nb, nd = _check(shapes, rays, g, o)
    assert nb > 1000


@pytest.mark.parametrize("accel", [abi.ACCEL_NONE, abi.ACCEL_BVH, abi.ACCEL_KDTREE])
def test_closest_modes_icosphere(accel, built_lib, orc):
    import ptgpu_pc_gb300 as pt
    shapes, lc, cam = scenes.icosphere_scene(level=4)
    rays = scenes.random_rays(20_000, seed=10)
    rays["o"] = rays["o"] * np.float32(40.0) + np.array([30, 20, 60], np.float32)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, lc)
        ctx.build(accel)
        g = ctx.trace_closest(rays)
    if accel == abi.ACCEL_KDTREE:
        acc = orc.make_accel(accel, kd=orc.KD(shapes))
    elif accel == abi.ACCEL_BVH:
        _, btn, btl, _ = orc.build_bvh(shapes)
        acc = orc.make_accel(accel, btn, btl)
    else:
        acc = orc.make_accel(accel)
    o = orc.trace_closest(shapes, rays, acc)
    nb, nd = _check(shapes, rays, g, o)
    assert nb > 1000


def test_closest_spheres_bruteforce(built_lib, orc):
    import ptgpu_pc_gb300 as pt
    shapes, lc, cam = scenes.cornell_spheres()
    rays = scenes.random_rays(20_000, seed=13)
    rays["o"] = rays["o"] * np.float32(40.0) + np.array([30, 20, 60], np.float32)
    for accel in (abi.ACCEL_NONE, abi.ACCEL_BVH, abi.ACCEL_KDTREE):
        with pt.Context(8, 8) as ctx:
            ctx.set_shapes(shapes, lc)
            ctx.build(accel)
            g = ctx.trace_closest(rays)
        o = orc.trace_closest(shapes, rays, orc.make_accel(abi.ACCEL_NONE))
        assert (g[2] == o[2]).all()
        assert (g[1][g[2] == 1] == o[1][o[2] == 1]).all()
        assert np.array_equal(g[0].view(np.uint32), o[0].view(np.uint32))


@pytest.mark.parametrize("accel", [abi.ACCEL_BVH, abi.ACCEL_KDTREE])
def test_binary_and_wide_traversal_agree(accel, built_lib, orc):
    """The 2-wide and the 4-wide node layouts give the same closest hits."""
    import ptgpu_pc_gb300 as pt
    shapes, lc, cam = scenes.icosphere_scene(level=5)
    rays = scenes.random_rays(20_000, seed=16)
    rays["o"] = rays["o"] * np.float32(40.0) + np.array([30, 20, 60], np.float32)
    out = []
    for flags in (0, abi.FLAG_WIDE_TRAVERSAL):
        with pt.Context(8, 8, flags=flags) as ctx:
            ctx.set_shapes(shapes, lc)
            ctx.build(accel)
            out.append(ctx.trace_closest(rays))
    assert np.array_equal(out[0][2], out[1][2])
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32))
    assert (out[0][1] == out[1][1]).mean() > 0.9999
