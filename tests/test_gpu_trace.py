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


def _check(shapes, rays, g, o, report=None, name=None):
    """The closest-hit rule: every ray whose hit lies at least 1e-6
    (barycentric) from the hit triangle's edges gets the same answer as the
    oracle: the same hit flag, the same shape id, t within 1e-5 relative.
    A ray is exempt only when the oracle's hit, or the GPU's where the two
    disagree, lies within 1e-6 of an edge (shared-edge rays)."""
    gt, gid, ghit = g
    ot, oid, ohit = o
    gh = (ghit == 1) & (gt < 1e20)
    oh = (ohit == 1) & (ot < 1e20)
    m_o = np.ones(len(rays))
    m_g = np.ones(len(rays))
    m_o[oh] = _barycentric_margin(shapes, oid[oh], rays[oh], ot[oh])
    m_g[gh] = _barycentric_margin(shapes, gid[gh], rays[gh], gt[gh])
    exempt = (oh & (m_o < EDGE)) | (gh & (m_g < EDGE))
    flag_bad = (gh != oh) & ~exempt
    both = gh & oh
    id_bad = both & (gid != oid) & ~exempt
    rel = np.zeros(len(rays))
    rel[both] = np.abs(gt[both].astype(np.float64) - ot[both]) / np.maximum(np.abs(ot[both]), 1e-30)
    t_bad = both & (gid == oid) & (rel > T_RTOL) & ~exempt
    if report is not None:
        report(name, rays=len(rays), hits=int(oh.sum()), exempt=int(exempt.sum()),
               id_equal_frac=float((gid[both] == oid[both]).mean()) if both.any() else 1.0,
               max_rel_t=float(rel[both & ~exempt].max()) if (both & ~exempt).any() else 0.0,
               flag_bad=int(flag_bad.sum()), id_bad=int(id_bad.sum()), t_bad=int(t_bad.sum()))
    assert not flag_bad.any(), "hit/miss differ on %d rays away from edges" % flag_bad.sum()
    assert not id_bad.any(), "%d id mismatches away from edges" % id_bad.sum()
    assert not t_bad.any(), "t differs beyond 1e-5 on %d rays (max %g)" % (t_bad.sum(), rel[t_bad].max())
    return int(both.sum()), int(((gid != oid) & both).sum())


def test_closest_config3_soup_1m(built_lib, orc, parity_report):
    """Config 3 at 1M triangles: the unit-cube soup and 2^20 of its rays
    (origins in [-0.5,1.5]^3, uniform directions); the oracle walks the
    GPU-built tree (byte-equal to the oracle's own build, test_gpu_lbvh)
    in the reference's order."""
    import ptgpu_pc_gb300 as pt
    shapes = scenes.triangle_soup(1 << 20, seed=5)
    rays = scenes.random_rays(1 << 20, seed=4)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, 0)
        ctx.build(abi.ACCEL_BVH)
        g = ctx.trace_closest(rays)
        btn, btl = ctx.get_bvh()
    o = orc.trace_closest(shapes, rays, orc.make_accel(abi.ACCEL_BVH, btn, btl, fast=True))
    nb, nd = _check(shapes, rays, g, o, parity_report, "closest_config3_soup1m_2^20rays")
    assert nb > 100_000


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
