"""The GPU KD-tree build (the default for PTGPU_ACCEL_KDTREE) against the
oracle's pointer tree (KDTree::build, KDTree.cpp:89-182, restated) node by
node at the config-2 size, and against the host build of the same algorithm
(PTGPU_FLAG_KD_HOST): the exported heap and shape list byte for byte where the
tree fits the int16 layout, and identical closest hits (t bit patterns, shape
ids) through either tree otherwise."""
import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _small_cases():
    flat = scenes.triangle_soup(3000, seed=21)
    for f in ("p1", "p2", "p3"):
        flat[f][:, 1] = 0.5                 # every midpoint equal on y
    dup = scenes.triangle_soup(2000, seed=22)
    dup[500:1500] = dup[500]                # many identical shapes
    return {"cornell": scenes.cornell_spheres()[0], "soup": scenes.triangle_soup(5000, seed=23),
            "ico3": scenes.icosphere_scene(level=3)[0], "flat": flat, "dup": dup,
            "one": scenes.triangle_soup(1, seed=24), "two": scenes.triangle_soup(2, seed=25),
            "three": scenes.triangle_soup(3, seed=26)}


def _kd(shapes, flags):
    import ptgpu_pc_gb300 as pt
    with pt.Context(8, 8, accel=abi.ACCEL_KDTREE) as ctx:
        ctx.set_shapes(shapes, 0)
        ctx.build(abi.ACCEL_KDTREE, flags)
        return ctx.get_kdtree()


@pytest.mark.parametrize("case", ["cornell", "soup", "ico3", "flat", "dup", "one", "two", "three"])
def test_gpu_kd_equals_host_kd(case, built_lib):
    shapes = _small_cases()[case]
    g_kng, g_kn = _kd(shapes, 0)
    h_kng, h_kn = _kd(shapes, abi.FLAG_KD_HOST)
    assert g_kng.tobytes() == h_kng.tobytes()
    assert np.array_equal(g_kn, h_kn)


@pytest.mark.parametrize("which", ["ico6", "soup200k"])
def test_gpu_kd_traces_like_host_kd(which, built_lib):
    import ptgpu_pc_gb300 as pt
    shapes = scenes.icosphere_scene(level=6)[0] if which == "ico6" else scenes.triangle_soup(200_000, seed=27)
    rays = scenes.random_rays(50_000, seed=28)
    if which == "ico6":                      # rays from inside the box toward the sphere
        rays["o"] = np.array([50.0, 40.0, 150.0], np.float32) + 20 * rays["o"]
    out, ms = [], []
    for flags in (0, abi.FLAG_KD_HOST):
        with pt.Context(8, 8, accel=abi.ACCEL_KDTREE) as ctx:
            ctx.set_shapes(shapes, 0)
            ctx.build(abi.ACCEL_KDTREE, flags)
            ms.append(ctx.last_build_ms())
            out.append(ctx.trace_closest(rays))
    (tg, ig, hg), (th, ih, hh) = out
    assert hg.sum() > 0
    assert np.array_equal(hg, hh)
    assert np.array_equal(tg.view(np.uint32), th.view(np.uint32))
    assert np.array_equal(ig, ih)


def _oracle_bfs(kd):
    """The oracle's pointer tree (nodes in creation order) renumbered
    breadth-first, as ptgpu_kd_node_wide records."""
    order, pos = [0], {0: 0}
    for nd in order:
        for c in (kd.left[nd], kd.right[nd]):
            if c >= 0:
                pos[c] = len(order)
                order.append(c)
    out = np.zeros(len(order), abi.KD_NODE_WIDE)
    for i, nd in enumerate(order):
        out[i]["leaf"] = kd.leaf[nd]
        out[i]["nLeft"] = pos[kd.left[nd]] if kd.left[nd] >= 0 else -1
        out[i]["nRight"] = pos[kd.right[nd]] if kd.right[nd] >= 0 else -1
        out[i]["bound"] = kd.box[nd]
        if kd.leaf[nd]:
            out[i]["min"], out[i]["max"] = kd.kmin[nd], kd.kmax[nd]
    out["nParent"] = -1
    for i in range(len(out)):
        for c in (out[i]["nLeft"], out[i]["nRight"]):
            if c >= 0:
                out[c]["nParent"] = i
    return out


@pytest.mark.parametrize("which", ["ico6", "soup100k", "cornell", "one"])
def test_gpu_kd_equals_oracle_tree(which, built_lib, orc, parity_report):
    """Config 2 (the level-6 icosphere scene, 81,934 shapes: 2^18 heap
    slots, beyond the int16 export) and others: every node's leaf flag, box,
    children and leaf range, and the kn shape order, equal to the oracle's
    pointer tree."""
    import ptgpu_pc_gb300 as pt
    shapes = {"ico6": lambda: scenes.icosphere_scene(level=6)[0],
              "soup100k": lambda: scenes.triangle_soup(100_000, seed=29),
              "cornell": lambda: scenes.cornell_spheres()[0],
              "one": lambda: scenes.triangle_soup(1, seed=30)}[which]()
    with pt.Context(8, 8, accel=abi.ACCEL_KDTREE) as ctx:
        ctx.set_shapes(shapes, 0)
        ctx.build(abi.ACCEL_KDTREE)
        nodes, kn = ctx.get_kdtree_wide()
    kd = orc.KD(shapes)
    want = _oracle_bfs(kd)
    parity_report("kd_tree_%s" % which, shapes=len(shapes), nodes=len(nodes), depth=kd.max_depth,
                  equal=bool(nodes.tobytes() == want.tobytes() and np.array_equal(kn, kd.kn)))
    assert len(nodes) == len(want)
    assert np.array_equal(nodes["leaf"], want["leaf"])
    assert np.array_equal(nodes["nLeft"], want["nLeft"])
    assert np.array_equal(nodes["nRight"], want["nRight"])
    assert np.array_equal(nodes["nParent"], want["nParent"])
    assert nodes["bound"].tobytes() == want["bound"].tobytes()
    assert np.array_equal(nodes["min"], want["min"]) and np.array_equal(nodes["max"], want["max"])
    assert np.array_equal(kn, kd.kn)
