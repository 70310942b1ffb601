"""The oracle restatement against golden vectors produced by the reference's
own code (tests/golden/make_golden.py over oracle/_ref).  CPU only."""
import ctypes
import os

import numpy as np
import pytest

from ptgpu_pc_gb300 import abi

G = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(G, name))


def test_rng_stream(orc):
    z = load("rng.npz")
    s0, s1 = ctypes.c_uint32(int(z["seed0"])), ctypes.c_uint32(int(z["seed1"]))
    vals = np.array([orc.lib().orc_get_random(ctypes.byref(s0), ctypes.byref(s1))
                     for _ in range(len(z["values"]))], np.float32)
    assert np.array_equal(vals.view(np.uint32), z["values"].view(np.uint32))
    assert [s0.value, s1.value] == list(z["final"])


def test_radix_tree_topology(orc):
    z = load("radix_tree.npz")
    btn_all = z["btn"].view(abi.BVH_NODE)
    btl_all = z["btl"].view(abi.BVH_NODE)
    oi = ol = 0
    for n in z["ns"]:
        n = int(n)
        btn, btl = orc.radix_tree(n)
        assert btn.tobytes() == btn_all[oi:oi + n - 1].tobytes(), n
        assert btl.tobytes() == btl_all[ol:ol + n].tobytes(), n
        oi += n - 1
        ol += n


@pytest.mark.parametrize("case", ["cornell", "ico2", "soup1000", "soup777"])
def test_clbvh(case, orc):
    z = load("clbvh.npz")
    shapes_in = z[case + "_in"].view(abi.SHAPE)
    s, btn, btl, srt = orc.build_bvh(shapes_in)
    ref_shapes = z[case + "_shapes"].view(abi.SHAPE)
    assert np.array_equal(s["morton_code"], ref_shapes["morton_code"])
    assert s["b"].tobytes() == ref_shapes["b"].tobytes()
    assert np.array_equal(s["index"], ref_shapes["index"])
    # the O(N) stable sort gives the bubble sort's permutation
    assert np.array_equal(srt, z[case + "_sorted"])
    assert np.array_equal(orc.sort_desc(s["morton_code"], bubble=True), z[case + "_sorted"])
    rbtn = z[case + "_btn"].view(abi.BVH_NODE)
    rbtl = z[case + "_btl"].view(abi.BVH_NODE)
    assert btl.tobytes() == rbtl.tobytes()
    for f in ("min", "max", "nShape", "leaf", "nLeft", "nRight", "nParent", "cost", "area"):
        assert np.array_equal(btn[f].view(np.uint32) if btn[f].dtype.kind == "f" else btn[f],
                              rbtn[f].view(np.uint32) if rbtn[f].dtype.kind == "f" else rbtn[f]), f
    n = len(shapes_in)
    if n % 2 == 0:
        # even N has no node with one leaf and one internal child, so the
        # reference's refit (run in order) gives the exact unions too
        assert btn["bound"].tobytes() == rbtn["bound"].tobytes()


@pytest.mark.parametrize("case", ["cornell", "ico2", "soup500"])
def test_kdtree(case, orc):
    z = load("kdtree.npz")
    shapes_in = z[case + "_in"].view(abi.SHAPE)
    kng, kn, st = orc.KD(shapes_in).heap()
    rkng = z[case + "_kng"].view(abi.KD_NODE)
    assert st == 0 and len(kng) == len(rkng)
    assert np.array_equal(kn, z[case + "_kn"])
    stack = [1]
    while stack:           # real nodes only; the reference leaves null slots unset
        p = stack.pop()
        a, b = kng[p], rkng[p]
        for f in ("leaf", "nLeft", "nRight", "nParent"):
            assert a[f] == b[f], (p, f)
        assert a["bound"].tobytes() == b["bound"].tobytes()
        if a["leaf"]:
            assert a["min"] == b["min"] and a["max"] == b["max"]
        else:
            stack += [int(a["nLeft"]), int(a["nRight"])]


def test_camera(orc):
    z = load("obj_model_scene.npz")
    cam = z["camera"].view(abi.CAMERA)[0]
    assert orc.update_camera(cam).tobytes() == z["camera_updated"].tobytes()


@pytest.mark.parametrize("accel", [0, 1, 2])
def test_intersect(accel, orc):
    z = load("obj_model_ref.npz")
    sh = load("obj_model_scene.npz")["shapes"].view(abi.SHAPE)
    rays = z["rays"].view(abi.RAY)
    if accel == 1:
        acc = orc.make_accel(1, z["bvh_btn"].view(abi.BVH_NODE), z["bvh_btl"].view(abi.BVH_NODE),
                             reference_leafness=True)
    elif accel == 2:
        acc = orc.make_accel(2, kd=orc.KD(sh))
    else:
        acc = orc.make_accel(0)
    t, ids, hit = orc.trace_closest(sh, rays, acc)
    assert np.array_equal(t.view(np.uint32), z["hit%d_t" % accel].view(np.uint32))
    assert np.array_equal(ids, z["hit%d_id" % accel])
    assert np.array_equal(hit, z["hit%d_hit" % accel])


@pytest.mark.parametrize("accel", [0, 1, 2])
def test_render_obj_model(accel, orc):
    """Bit-exact with the reference's RadianceGPU compiled by g++ (which
    evaluates the light sampler's two random arguments right to left)."""
    z = load("obj_model_ref.npz")
    sc = load("obj_model_scene.npz")
    sh = sc["shapes"].view(abi.SHAPE)
    lc = int(sc["light_cnt"])
    cam = z["camera"].view(abi.CAMERA)[0]
    w, h = 40, 30
    if accel == 1:
        acc = orc.make_accel(1, z["bvh_btn"].view(abi.BVH_NODE), z["bvh_btl"].view(abi.BVH_NODE),
                             reference_leafness=True)
    elif accel == 2:
        acc = orc.make_accel(2, kd=orc.KD(sh))
    else:
        acc = orc.make_accel(0)
    col, pix, sd = orc.render(sh, lc, cam, w, h, z["seeds"], 2, accel=acc, arg_order_rtl=True)
    assert col.tobytes() == z["render%d_colors" % accel].tobytes()
    assert np.array_equal(pix, z["render%d_pixels" % accel])
    assert np.array_equal(sd, z["render%d_seeds" % accel])


def test_render_cornell_spheres(orc):
    z = load("cornell_ref.npz")
    sh = z["shapes"].view(abi.SHAPE)
    cam = z["camera"].view(abi.CAMERA)[0]
    col, pix, sd = orc.render(sh, 1, cam, 32, 32, z["seeds"], 3, arg_order_rtl=True)
    assert col.tobytes() == z["colors"].tobytes()
    assert np.array_equal(pix, z["pixels"])
    assert np.array_equal(sd, z["seeds_out"])


def test_treelet_rounds_lower_sah_and_keep_leaves(orc):
    """Each treelet round keeps every leaf exactly once and never raises the
    SAH cost; later rounds start from the tree the earlier ones left."""
    from ptgpu_pc_gb300 import scenes
    shapes = scenes.triangle_soup(3000, seed=31)
    _, btn, btl, _ = orc.build_bvh(shapes)
    costs = [orc.sah_cost(btn, btl)]
    for k in (1, 2, 3):
        b, l = orc.treelet_optimize(btn, btl, k)
        costs.append(orc.sah_cost(b, l))
        # leaf children of the internal nodes: every leaf once
        kids = np.concatenate([b["nLeft"][b["min"] == b["nLeft"]], b["nRight"][b["max"] == b["nRight"]]])
        assert np.array_equal(np.sort(kids), np.arange(len(shapes)))
    assert costs[1] <= costs[0] and costs[2] <= costs[1] + 1e-9 and costs[3] <= costs[2] + 1e-9
    b2, l2 = orc.treelet_optimize(*orc.treelet_optimize(btn, btl, 1), 1)
    b3, l3 = orc.treelet_optimize(btn, btl, 2)
    assert b2["nLeft"].tobytes() == b3["nLeft"].tobytes()
