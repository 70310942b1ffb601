"""Generates the golden fixtures in tests/golden/ from the reference's own
code (oracle/_ref: CLBVH.cpp, KDTree.cpp, displayfunc.cpp, BVH.cl and
rendering_kernel.cl compiled on the CPU by oracle/ref/build_ref.sh).

Run here, where the reference tree is available:
    python tests/golden/make_golden.py
The outputs are small .npz files; the tests compare the oracle restatement
against them, so the oracle stays pinned on machines without the reference.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from ptgpu_pc_gb300 import abi, scenes  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


def raw(a):
    return np.ascontiguousarray(a).view(np.uint8)


def main():
    oracle.build()
    oracle.build_ref()
    R = oracle.ref()
    import ctypes
    # 1. RNG stream
    s0, s1 = ctypes.c_uint32(12345), ctypes.c_uint32(678)
    seq = np.array([R.ref_get_random(ctypes.byref(s0), ctypes.byref(s1)) for _ in range(4096)], np.float32)
    save("rng.npz", seed0=np.uint32(12345), seed1=np.uint32(678), values=seq,
         final=np.array([s0.value, s1.value], np.uint32))
    # 2. radix tree topology for every N in 2..600 plus a few larger ones
    ns = list(range(2, 601)) + [1023, 1024, 1025, 4095, 4096, 4097]
    btn_all, btl_all = [], []
    for n in ns:
        btn, btl = oracle.ref_radix_tree(n)
        btn_all.append(raw(btn).reshape(-1)); btl_all.append(raw(btl).reshape(-1))
    save("radix_tree.npz", ns=np.array(ns, np.int32), btn=np.concatenate(btn_all),
         btl=np.concatenate(btl_all))
    # 3. CLBVH on small scenes: Morton codes, bubble-sort order, full trees
    cases = {"cornell": scenes.cornell_spheres()[0], "ico2": scenes.icosphere_scene(level=2)[0],
             "soup1000": scenes.triangle_soup(1000, seed=21), "soup777": scenes.triangle_soup(777, seed=22)}
    out = {}
    for name, sh in cases.items():
        s_ref, btn, btl = oracle.ref_clbvh(sh, refit=True)
        out[name + "_in"] = raw(sh)
        out[name + "_shapes"] = raw(s_ref)
        out[name + "_sorted"] = oracle.ref_bubblesort(s_ref)
        out[name + "_btn"] = raw(btn)
        out[name + "_btl"] = raw(btl)
    save("clbvh.npz", **out)
    # 4. KD trees (heap layout) on small scenes
    out = {}
    for name, sh in {"cornell": scenes.cornell_spheres()[0], "ico2": scenes.icosphere_scene(level=2)[0],
                     "soup500": scenes.triangle_soup(500, seed=23)}.items():
        kng, kn = oracle.ref_kd_build(sh)
        out[name + "_in"] = raw(sh)
        out[name + "_kng"] = raw(kng)
        out[name + "_kn"] = kn
    save("kdtree.npz", **out)
    # 5. the reference scene file (scenes/obj-model.txt + models/*.obj) as
    #    loaded by the reference loader, and its UpdateCamera
    st, sh, lc, cam, wl = oracle.ref_read_scene("scenes/obj-model.txt", 40, 30)
    assert st == 0
    cam_u = oracle.ref_update_camera(cam)
    save("obj_model_scene.npz", shapes=raw(sh), light_cnt=np.int32(lc), camera=raw(cam),
         camera_updated=raw(cam_u), walllight=np.int32(wl))
    # 6. closest hits (Intersect, all three modes) and renders (RadianceGPU)
    #    on the obj-model scene, seeds from SplitMix64(5)
    rays = scenes.random_rays(3000, seed=31)
    rays["o"] = rays["o"] * np.float32(40.0) + np.array([-20, 30, 20], np.float32)
    _, btn, btl, _ = oracle.build_bvh(sh)
    kng, kn = oracle.ref_kd_build(sh)
    w, h = 40, 30
    seeds = oracle.make_seeds(5, 2 * w * h)
    cam_r = np.array(cam, abi.CAMERA); cam_r["width"], cam_r["height"] = w, h
    cam_r = oracle.ref_update_camera(cam_r)
    out = dict(rays=raw(rays), seeds=seeds, bvh_btn=raw(btn), bvh_btl=raw(btl), kng=raw(kng), kn=kn,
               camera=raw(cam_r))
    for accel in (0, 1, 2):
        t, ids, hit = oracle.ref_intersect(accel, sh, rays, btn=btn, btl=btl, kng=kng, kn=kn)
        out["hit%d_t" % accel], out["hit%d_id" % accel], out["hit%d_hit" % accel] = t, ids, hit
        col, pix, sd = oracle.ref_render(accel, sh, lc, cam_r, w, h, seeds, 2, btn=btn, btl=btl,
                                         kng=kng, kn=kn)
        out["render%d_colors" % accel] = raw(col)
        out["render%d_pixels" % accel] = pix
        out["render%d_seeds" % accel] = sd
    save("obj_model_ref.npz", **out)
    # 7. the 9-sphere Cornell scene rendered by the reference (no accel)
    shapes, lc, cam = scenes.cornell_spheres()
    w, h = 32, 32
    seeds = oracle.make_seeds(1, 2 * w * h)
    c = np.array(cam, abi.CAMERA); c["width"], c["height"] = w, h
    c = oracle.ref_update_camera(c)
    col, pix, sd = oracle.ref_render(0, shapes, lc, c, w, h, seeds, 3)
    save("cornell_ref.npz", shapes=raw(shapes), camera=raw(c), seeds=seeds, colors=raw(col),
         pixels=pix, seeds_out=sd)


if __name__ == "__main__":
    main()
