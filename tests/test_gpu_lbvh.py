"""GPU LBVH build vs the oracle (CLBVH + BVH.cl restated): Morton keys, the
sorted permutation, and the btn/btl arrays byte for byte."""
import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _gpu_build(shapes, light_cnt=0):
    import ptgpu_pc_gb300 as pt
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, light_cnt)
        ctx.build(abi.ACCEL_BVH)
        btn, btl = ctx.get_bvh()
        out = ctx.get_shapes()
        ms = ctx.last_build_ms()
    return out, btn, btl, ms


def _compare(shapes, orc):
    g_shapes, g_btn, g_btl, _ = _gpu_build(shapes)
    o_shapes, o_btn, o_btl, o_sorted = orc.build_bvh(shapes)
    assert (g_shapes["morton_code"] == o_shapes["morton_code"]).all()
    assert (g_shapes["index"] == o_shapes["index"]).all()
    assert g_shapes["b"].tobytes() == o_shapes["b"].tobytes()
    assert (g_btl["nShape"] == o_sorted).all()
    assert g_btl.tobytes() == o_btl.tobytes()
    assert g_btn.tobytes() == o_btn.tobytes()


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 13, 100, 1000, 1023, 1024, 1025, 2047, 4097, 12345])
def test_lbvh_soup_small(n, built_lib, orc):
    _compare(scenes.triangle_soup(n, seed=n), orc)


def test_lbvh_cornell_spheres(built_lib, orc):
    _compare(scenes.cornell_spheres()[0], orc)


def test_lbvh_icosphere_scene(built_lib, orc):
    _compare(scenes.icosphere_scene(level=6)[0], orc)


def test_lbvh_duplicate_keys_and_flat_axis(built_lib, orc):
    # every centroid in the z = 0 plane (flat axis: max == min -> code bits 0)
    # and many identical triangles (duplicate keys: the sort must stay stable)
    s = scenes.triangle_soup(5000, seed=11)
    for f in ("p1", "p2", "p3"):
        s[f][:, 2] = 0.0
    s[1000:3000] = s[1000]
    _compare(s, orc)


def test_lbvh_negative_coordinates(built_lib, orc):
    # all centroids negative: the reference's FLT_MIN initial maximum is kept
    s = scenes.triangle_soup(3000, seed=12)
    for f in ("p1", "p2", "p3"):
        s[f] -= 10.0
    _compare(s, orc)


def test_lbvh_mixed_spheres_triangles(built_lib, orc):
    # spheres shuffled among triangles: whole warps of 32 shapes take both
    # the sphere and the triangle bound and centroid forms
    rng = np.random.default_rng(21)
    m = 6000
    sph = abi.spheres(rng.uniform(0.001, 0.02, m), rng.random((m, 3)), np.zeros((m, 3)),
                      np.full((m, 3), 0.5), np.zeros(m, np.int32))
    tri = scenes.triangle_soup(14001, seed=21)
    s = np.zeros(len(tri) + m, abi.SHAPE)
    s[:len(tri)] = tri
    s[len(tri):] = sph
    _compare(s[rng.permutation(len(s))], orc)


@pytest.mark.parametrize("n", [1 << 20, (1 << 20) + 7, 1 << 22])
def test_lbvh_1m(n, built_lib, orc):
    """Config 3's soups (1M and 4M triangles) and an odd size: Morton keys,
    sorted order and both node arrays byte for byte."""
    _compare(scenes.triangle_soup(n, seed=5), orc)


@pytest.mark.parametrize("n", [1 << 22, (1 << 24) + 7])
def test_lbvh_large_properties(n, built_lib):
    """4M and 16.7M triangles (the second climbs above 2^24 leaves with
    arrival counters): size-independent checks -- each shape exactly once in
    the leaves, keys non-increasing along the leaves, stable ties, every
    internal bound equal to the union of its children, the children's ranges
    splitting the parent's at nLeft, and parents pointing back."""
    shapes = scenes.triangle_soup(n, seed=6)
    g_shapes, btn, btl, ms = _gpu_build(shapes)
    del shapes
    order = btl["nShape"]
    assert np.array_equal(np.sort(order), np.arange(n))
    keys = g_shapes["morton_code"][order]
    assert (keys[:-1] >= keys[1:]).all()
    # stability: equal keys keep index order
    eq = keys[:-1] == keys[1:]
    assert (order[:-1][eq] < order[1:][eq]).all()
    del keys, eq, order, g_shapes
    ll = btn["nLeft"] == btn["min"]
    rl = btn["nRight"] == btn["max"]
    lb = np.where(ll[:, None], btl["bound"][btn["nLeft"]], btn["bound"][np.minimum(btn["nLeft"], n - 2)])
    rb = np.where(rl[:, None], btl["bound"][btn["nRight"]], btn["bound"][np.minimum(btn["nRight"], n - 2)])
    mins = np.where(lb[:, 0::2] < rb[:, 0::2], lb[:, 0::2], rb[:, 0::2])
    maxs = np.where(lb[:, 1::2] > rb[:, 1::2], lb[:, 1::2], rb[:, 1::2])
    assert np.array_equal(btn["bound"][:, 0::2], mins)
    assert np.array_equal(btn["bound"][:, 1::2], maxs)
    del lb, rb, mins, maxs
    idx = np.arange(n - 1, dtype=np.int32)
    nl, nr = btn["nLeft"], btn["nRight"]
    assert np.array_equal(nr, nl + 1)
    assert btn["min"][0] == 0 and btn["max"][0] == n - 1
    # internal children: ranges [min, nLeft] and [nRight, max], parent = this node
    li = ~ll
    assert np.array_equal(btn["min"][nl[li]], btn["min"][li])
    assert np.array_equal(btn["max"][nl[li]], nl[li])
    assert np.array_equal(btn["nParent"][nl[li]], idx[li])
    ri = ~rl
    assert np.array_equal(btn["min"][nr[ri]], nr[ri])
    assert np.array_equal(btn["max"][nr[ri]], btn["max"][ri])
    assert np.array_equal(btn["nParent"][nr[ri]], idx[ri])
    assert np.array_equal(btl["nParent"][nl[ll]], idx[ll])
    assert np.array_equal(btl["nParent"][nr[rl]], idx[rl])
    assert ms > 0


@pytest.mark.parametrize("case,sweeps", [("ico4", 1), ("soup", 1), ("cornell", 1), ("odd", 1),
                                         ("ico4", 3), ("soup", 2), ("odd", 3), ("tiny", 3),
                                         ("ico6", 3)])
def test_treelet_matches_oracle(case, sweeps, built_lib, orc):
    """GPU treelet restructuring == the oracle's sequential restatement, byte
    for byte, after one or several rounds; the SAH cost drops."""
    import ptgpu_pc_gb300 as pt
    shapes = {"ico4": lambda: scenes.icosphere_scene(level=4)[0],
              "ico6": lambda: scenes.icosphere_scene(level=6)[0],
              "soup": lambda: scenes.triangle_soup(30000, seed=4),
              "cornell": lambda: scenes.cornell_spheres()[0],
              "odd": lambda: scenes.triangle_soup(4097, seed=5),
              "tiny": lambda: scenes.triangle_soup(5, seed=6)}[case]()
    flags = abi.FLAG_TREELET | (abi.treelet_sweeps(sweeps) if sweeps > 1 else 0)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, 0)
        ctx.build(abi.ACCEL_BVH, flags)
        g_btn, g_btl = ctx.get_bvh()
    _, btn, btl, _ = orc.build_bvh(shapes)
    o_btn, o_btl = orc.treelet_optimize(btn, btl, sweeps)
    assert g_btl.tobytes() == o_btl.tobytes()
    assert g_btn.tobytes() == o_btn.tobytes()
    if len(shapes) > 2:
        assert orc.sah_cost(g_btn, g_btl) <= orc.sah_cost(btn, btl) + 1e-9


def test_treelet_closest_hits_unchanged(built_lib, orc):
    import ptgpu_pc_gb300 as pt
    shapes = scenes.triangle_soup(100_000, seed=14)
    rays = scenes.random_rays(30_000, seed=15)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, 0)
        ctx.build(abi.ACCEL_BVH)
        a = ctx.trace_closest(rays)
        ctx.build(abi.ACCEL_BVH, abi.FLAG_TREELET)
        b = ctx.trace_closest(rays)
    assert np.array_equal(a[2], b[2])
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
    assert (a[1] == b[1]).mean() > 0.9999
