"""CPU oracle for the PTGPU_PC hot path -- TEST INFRASTRUCTURE ONLY.

Python bindings over oracle/ptgpu_oracle.c (a C restatement of the reference
algorithms) and, where the reference tree was available when the library was
built, over oracle/_ref/libptgpu_ref.so (the reference's own sources compiled
on the CPU).  Only the tests, the smoke check and the benchmark's CPU-baseline
leg import this package; the GPU library never does.
"""
import ctypes
import os
import subprocess

import numpy as np

from ptgpu_pc_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libptgpu_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libptgpu_ref.so")
# The reference tree is found only through PTGPU_REFERENCE_DIR; without it
# the reference build (oracle/_ref) is skipped and the tests that need it
# skip with that reason.
REFERENCE_DIR = os.environ.get("PTGPU_REFERENCE_DIR", "")

_lib = None
_ref = None


def build(force=False):
    """Compiles the C restatement (gcc, no FP contraction, OpenMP)."""
    src = os.path.join(HERE, "ptgpu_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(os.path.join(HERE, "ptgpu_oracle.h"))):
        return LIB_PATH
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
           "-shared", "-std=gnu11", "-o", LIB_PATH, src, "-lm"]
    subprocess.check_call(cmd)
    return LIB_PATH


def build_ref():
    """Builds oracle/_ref from the reference tree when PTGPU_REFERENCE_DIR
    names one."""
    if not REFERENCE_DIR or not os.path.isfile(os.path.join(REFERENCE_DIR, "include", "BVH.cl")):
        return None
    subprocess.check_call(["bash", os.path.join(HERE, "ref", "build_ref.sh")],
                          stdout=subprocess.DEVNULL)
    return REF_LIB_PATH


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, i32, f32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_float
        L.orc_get_random.restype = f32
        L.orc_get_random.argtypes = [vp, vp]
        L.orc_make_seeds.argtypes = [ctypes.c_uint64, vp, u32]
        L.orc_update_camera.argtypes = [vp]
        L.orc_generate_camera_ray.argtypes = [vp, vp, vp, i32, i32, i32, i32, vp]
        L.orc_trace_closest.argtypes = [vp, u32, vp, vp, u32, vp, vp, vp, vp, i32]
        L.orc_shadow_batch.argtypes = [vp, u32, vp, vp, vp, u32, vp, i32]
        L.orc_render_pass.argtypes = [vp, u32, u32, vp, i32, i32, vp, i32, i32, i32,
                                      vp, vp, vp, i32, i32, i32, i32, i32]
        L.orc_lbvh_morton.argtypes = [vp, u32]
        L.orc_sort_desc_stable.argtypes = [vp, u32, vp]
        L.orc_bubblesort_desc.argtypes = [vp, u32, vp]
        L.orc_radix_tree.argtypes = [u32, vp, vp]
        L.orc_refit.argtypes = [vp, u32, vp, vp, vp]
        L.orc_build_bvh.restype = i32
        L.orc_build_bvh.argtypes = [vp, u32, vp, vp, vp]
        L.orc_sah_cost.restype = ctypes.c_double
        L.orc_sah_cost.argtypes = [u32, vp, vp]
        L.orc_treelet_optimize.argtypes = [u32, vp, vp]
        L.orc_treelet_optimize_sweeps.argtypes = [u32, vp, vp, ctypes.c_int]
        L.orc_kd_build.argtypes = [vp, u32, ctypes.POINTER(KdTree)]
        L.orc_kd_free.argtypes = [ctypes.POINTER(KdTree)]
        L.orc_kd_heap.restype = i32
        L.orc_kd_heap.argtypes = [ctypes.POINTER(KdTree), vp, i32, vp]
        L.orc_to_int.restype = u32
        L.orc_set_portable_trig.argtypes = [i32]
        L.orc_set_rr_depth.argtypes = [i32]
        L.orc_set_reference_cost.argtypes = [i32]
        L.orc_to_int.argtypes = [f32]
        _lib = L
    return _lib


class Counters(ctypes.Structure):
    _fields_ = [("node_visits", ctypes.c_uint64), ("prim_tests", ctypes.c_uint64),
                ("rays", ctypes.c_uint64)]


class Accel(ctypes.Structure):
    _fields_ = [("accel", ctypes.c_int32), ("btn", ctypes.c_void_p), ("btl", ctypes.c_void_p),
                ("bvh_reference_leafness", ctypes.c_int32),
                ("kd_leaf", ctypes.c_void_p), ("kd_left", ctypes.c_void_p),
                ("kd_right", ctypes.c_void_p), ("kd_box", ctypes.c_void_p),
                ("kd_min", ctypes.c_void_p), ("kd_max", ctypes.c_void_p),
                ("kd_kn", ctypes.c_void_p), ("kd_root", ctypes.c_int32),
                ("shadow_accel", ctypes.c_int32), ("cull_closest", ctypes.c_int32)]


class KdTree(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int32), ("cap_nodes", ctypes.c_int32),
                ("leaf", ctypes.c_void_p), ("left", ctypes.c_void_p),
                ("right", ctypes.c_void_p), ("depth", ctypes.c_void_p),
                ("box", ctypes.c_void_p), ("kmin", ctypes.c_void_p),
                ("kmax", ctypes.c_void_p), ("kn", ctypes.c_void_p),
                ("kn_cnt", ctypes.c_int32), ("kn_cap", ctypes.c_int32),
                ("max_depth", ctypes.c_int32), ("szbuf", ctypes.c_int32)]


def _np_from(ptr, count, dtype):
    if count == 0:
        return np.zeros(0, dtype)
    buf = (ctypes.c_char * (count * np.dtype(dtype).itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype, count=count).copy()


class KD:
    """Pointer-tree KD build (KDTree::build) held as numpy arrays."""

    def __init__(self, shapes):
        self.shapes = abi.as_struct(shapes, abi.SHAPE)
        t = KdTree()
        lib().orc_kd_build(_ptr(self.shapes), len(self.shapes), ctypes.byref(t))
        n = t.n_nodes
        self.n_nodes = n
        self.leaf = _np_from(t.leaf, n, np.int32)
        self.left = _np_from(t.left, n, np.int32)
        self.right = _np_from(t.right, n, np.int32)
        self.depth = _np_from(t.depth, n, np.int32)
        self.box = _np_from(t.box, n * 6, np.float32).reshape(n, 6)
        self.kmin = _np_from(t.kmin, n, np.int32)
        self.kmax = _np_from(t.kmax, n, np.int32)
        self.kn = _np_from(t.kn, t.kn_cnt, np.int32)
        self.max_depth = t.max_depth
        self.szbuf = t.szbuf
        self._t = t

    def heap(self):
        """KDTree::getTrees layout; returns (kng, kn, status)."""
        size = 1 << (self.max_depth + 1)
        kng = np.zeros(size, abi.KD_NODE)
        kn = np.zeros(max(self.szbuf, 1), np.int32)
        st = lib().orc_kd_heap(ctypes.byref(self._t), _ptr(kng), size, _ptr(kn))
        return kng, kn[: self.szbuf], st

    def __del__(self):
        try:
            lib().orc_kd_free(ctypes.byref(self._t))
        except Exception:
            pass


def make_accel(accel, btn=None, btl=None, kd=None, reference_leafness=False, fast=False):
    """fast: two oracle-side speed-ups for scenes where the reference's loops
    are too slow on the CPU.  The renderer's shadow queries (IntersectP: any
    shape but the last hit at 0 < d < maxt) go through the tree instead of the
    brute-force loop, and the closest-hit walk skips boxes that cannot hold a
    better hit (same visit order, same results).  The CPU tests compare both
    with the plain forms (shadow_batch, trace_closest)."""
    a = Accel()
    a.accel = accel
    a.shadow_accel = 1 if fast else 0
    a.cull_closest = 1 if fast else 0
    keep = []
    if accel == abi.ACCEL_BVH:
        a.btn, a.btl = _ptr(btn), _ptr(btl)
        a.bvh_reference_leafness = 1 if reference_leafness else 0
        keep += [btn, btl]
    elif accel == abi.ACCEL_KDTREE:
        a.kd_leaf, a.kd_left, a.kd_right = _ptr(kd.leaf), _ptr(kd.left), _ptr(kd.right)
        a.kd_box, a.kd_min, a.kd_max, a.kd_kn = _ptr(kd.box), _ptr(kd.kmin), _ptr(kd.kmax), _ptr(kd.kn)
        a.kd_root = 0
        keep += [kd]
    a._keep = keep
    return a


def make_seeds(master, count):
    s = np.zeros(count, np.uint32)
    lib().orc_make_seeds(master, _ptr(s), count)
    return s


def update_camera(cam):
    c = np.array(cam, abi.CAMERA).reshape(1)
    lib().orc_update_camera(_ptr(c))
    return c[0]


def trace_closest(shapes, rays, accel=None, threads=0, count=False):
    shapes = abi.as_struct(shapes, abi.SHAPE)
    rays = np.ascontiguousarray(rays)
    n = len(rays)
    t = np.zeros(n, np.float32)
    ids = np.zeros(n, np.uint32)
    hit = np.zeros(n, np.int32)
    cnt = Counters()
    a = accel if accel is not None else make_accel(abi.ACCEL_NONE)
    lib().orc_trace_closest(_ptr(shapes), len(shapes), ctypes.byref(a), _ptr(rays), n,
                            _ptr(t), _ptr(ids), _ptr(hit),
                            ctypes.byref(cnt) if count else None, threads)
    if count:
        return t, ids, hit, cnt
    return t, ids, hit


def shadow_batch(shapes, rays, maxt, accel=None, threads=0):
    """IntersectP for each ray; brute force unless accel.shadow_accel."""
    shapes = abi.as_struct(shapes, abi.SHAPE)
    rays = np.ascontiguousarray(rays)
    maxt = np.ascontiguousarray(maxt, np.float32)
    occ = np.zeros(len(rays), np.int32)
    a = accel if accel is not None else make_accel(abi.ACCEL_NONE)
    lib().orc_shadow_batch(_ptr(shapes), len(shapes), ctypes.byref(a), _ptr(rays), _ptr(maxt),
                           len(rays), _ptr(occ), threads)
    return occ


def render(shapes, light_cnt, cam, w, h, seeds, passes, accel=None, max_depth=6,
           arg_order_rtl=False, colors=None, start_sample=0, threads=0, rows=None,
           portable_trig=False, cols=None, rr_depth=0, reference_cost=False):
    """Runs `passes` RadianceGPU passes; returns (colors, pixels, seeds).
    portable_trig selects the GPU library's own sin/cos instead of libm;
    rr_depth > 0 adds the opt-in throughput Russian roulette;
    reference_cost rescans the shapes for emitters at every diffuse hit, as
    the reference does (same result, the reference's cost)."""
    lib().orc_set_portable_trig(1 if portable_trig else 0)
    lib().orc_set_rr_depth(int(rr_depth))
    lib().orc_set_reference_cost(1 if reference_cost else 0)
    shapes = abi.as_struct(shapes, abi.SHAPE)
    cam = np.array(cam, abi.CAMERA).reshape(1)
    seeds = np.array(seeds, np.uint32, copy=True)
    if colors is None:
        colors = np.zeros(w * h, abi.VEC)
    pixels = np.zeros(w * h, np.uint32)
    a = accel if accel is not None else make_accel(abi.ACCEL_NONE)
    r0, r1 = rows if rows is not None else (0, h)
    c0, c1 = cols if cols is not None else (0, w)
    for p in range(passes):
        lib().orc_render_pass(_ptr(shapes), len(shapes), light_cnt, ctypes.byref(a), max_depth,
                              1 if arg_order_rtl else 0, _ptr(cam), w, h, start_sample + p,
                              _ptr(colors), _ptr(pixels), _ptr(seeds), r0, r1, c0, c1, threads)
    return colors, pixels, seeds


def lbvh_morton(shapes):
    s = np.array(shapes, abi.SHAPE, copy=True)
    lib().orc_lbvh_morton(_ptr(s), len(s))
    return s


def sort_desc(keys, bubble=False):
    keys = np.ascontiguousarray(keys, np.uint32)
    out = np.zeros(len(keys), np.int32)
    (lib().orc_bubblesort_desc if bubble else lib().orc_sort_desc_stable)(_ptr(keys), len(keys), _ptr(out))
    return out


def radix_tree(n):
    btn = np.zeros(max(n - 1, 0), abi.BVH_NODE)
    btl = np.zeros(n, abi.BVH_NODE)
    lib().orc_radix_tree(n, _ptr(btn), _ptr(btl))
    return btn, btl


def build_bvh(shapes):
    """Full LBVH build; returns (shapes with b/index/morton, btn, btl, sorted)."""
    s = np.array(shapes, abi.SHAPE, copy=True)
    n = len(s)
    btn = np.zeros(max(n - 1, 0), abi.BVH_NODE)
    btl = np.zeros(n, abi.BVH_NODE)
    srt = np.zeros(n, np.int32)
    lib().orc_build_bvh(_ptr(s), n, _ptr(btn), _ptr(btl), _ptr(srt))
    return s, btn, btl, srt


def sah_cost(btn, btl):
    return lib().orc_sah_cost(len(btl), _ptr(btn), _ptr(btl))


def treelet_optimize(btn, btl, sweeps=1):
    btn = btn.copy(); btl = btl.copy()
    lib().orc_treelet_optimize_sweeps(len(btl), _ptr(btn), _ptr(btl), sweeps)
    return btn, btl


def to_int(x):
    return lib().orc_to_int(float(x))


# --------------------------------------------------------------------------
# reference library (only where the reference tree was present at build time)
# --------------------------------------------------------------------------
def ref_available():
    return os.path.exists(REF_LIB_PATH)


def ref():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB_PATH):
            raise RuntimeError("oracle/_ref not built (the reference tree is absent)")
        R = ctypes.CDLL(REF_LIB_PATH)
        vp, i32, u32, f32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_float
        R.ref_get_random.restype = f32
        R.ref_get_random.argtypes = [vp, vp]
        R.ref_radix_tree.argtypes = [i32, vp, vp]
        R.ref_render_pass.argtypes = [i32, vp, vp, vp, vp, u32, u32, vp, vp, vp, i32, vp, i32,
                                      i32, i32, i32, vp]
        R.ref_intersect.argtypes = [i32, vp, u32, vp, vp, vp, i32, vp, i32, vp, i32, vp, vp, vp]
        R.ref_intersect_p.restype = i32
        R.ref_intersect_p.argtypes = [vp, u32, vp, f32]
        R.ref_generate_camera_ray.argtypes = [vp, vp, vp, i32, i32, i32, i32, vp]
        R.ref_clbvh.argtypes = [vp, i32, vp, vp, i32]
        R.ref_bubblesort.argtypes = [vp, i32, vp]
        R.ref_kd_build.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(i32),
                                   ctypes.POINTER(vp), ctypes.POINTER(i32)]
        R.ref_free.argtypes = [vp]
        R.ref_read_scene.restype = i32
        R.ref_read_scene.argtypes = [ctypes.c_char_p, i32, i32, ctypes.POINTER(vp),
                                     ctypes.POINTER(u32), ctypes.POINTER(u32), vp,
                                     ctypes.POINTER(i32)]
        R.ref_update_camera.argtypes = [vp]
        for a in (0, 1, 2):
            fn = getattr(R, "ref_cpu_render_acc%d" % a)
            fn.argtypes = [vp, vp, u32, u32, vp, vp, vp, i32, vp, i32, i32, i32, i32, i32, i32,
                           vp, vp, i32]
        _ref = R
    return _ref


def ref_clbvh(shapes, refit=False):
    s = np.array(shapes, abi.SHAPE, copy=True)
    n = len(s)
    btn = np.zeros(max(n - 1, 1), abi.BVH_NODE)
    btl = np.zeros(n, abi.BVH_NODE)
    ref().ref_clbvh(_ptr(s), n, _ptr(btn), _ptr(btl), 1 if refit else 0)
    return s, btn[: max(n - 1, 0)], btl


def ref_bubblesort(shapes_with_codes):
    s = np.array(shapes_with_codes, abi.SHAPE, copy=True)
    out = np.zeros(len(s), np.int32)
    ref().ref_bubblesort(_ptr(s), len(s), _ptr(out))
    return out


def ref_radix_tree(n):
    btn = np.zeros(max(n - 1, 1), abi.BVH_NODE)
    btl = np.zeros(n, abi.BVH_NODE)
    ref().ref_radix_tree(n, _ptr(btn), _ptr(btl))
    return btn[: max(n - 1, 0)], btl


def ref_kd_build(shapes):
    s = np.array(shapes, abi.SHAPE, copy=True)
    pk, pn = ctypes.c_void_p(), ctypes.c_void_p()
    ck, cn = ctypes.c_int32(), ctypes.c_int32()
    ref().ref_kd_build(_ptr(s), len(s), ctypes.byref(pk), ctypes.byref(ck), ctypes.byref(pn),
                       ctypes.byref(cn))
    kng = _np_from(pk.value, ck.value, abi.KD_NODE)
    kn = _np_from(pn.value, cn.value, np.int32)
    ref().ref_free(pk); ref().ref_free(pn)
    return kng, kn


def ref_read_scene(path, w, h):
    ps = ctypes.c_void_p()
    n, lc = ctypes.c_uint32(), ctypes.c_uint32()
    cam = np.zeros(1, abi.CAMERA)
    wl = ctypes.c_int32()
    cwd = os.getcwd()
    try:
        os.chdir(REFERENCE_DIR)  # the scene file names models relative to the tree
        st = ref().ref_read_scene(path.encode(), w, h, ctypes.byref(ps), ctypes.byref(n),
                                  ctypes.byref(lc), _ptr(cam), ctypes.byref(wl))
    finally:
        os.chdir(cwd)
    shapes = _np_from(ps.value, n.value, abi.SHAPE) if ps.value else np.zeros(0, abi.SHAPE)
    return st, shapes, lc.value, cam[0], wl.value


def ref_update_camera(cam):
    c = np.array(cam, abi.CAMERA).reshape(1)
    ref().ref_update_camera(_ptr(c))
    return c[0]


def ref_render(accel, shapes, light_cnt, cam, w, h, seeds, passes, btn=None, btl=None,
               kng=None, kn=None):
    shapes = np.array(shapes, abi.SHAPE, copy=True)
    cam = np.array(cam, abi.CAMERA).reshape(1)
    seeds = np.array(seeds, np.uint32, copy=True)
    colors = np.zeros(w * h, abi.VEC)
    pixels = np.zeros(w * h, np.int32)
    kng_cnt = len(kng) if kng is not None else 0
    kn_cnt = len(kn) if kn is not None else 0
    for p in range(passes):
        ref().ref_render_pass(accel, _ptr(colors), _ptr(seeds), _ptr(cam), _ptr(shapes),
                              len(shapes), light_cnt, _ptr(btn), _ptr(btl), _ptr(kng), kng_cnt,
                              _ptr(kn), kn_cnt, w, h, p, _ptr(pixels))
    return colors, pixels.view(np.uint32), seeds


def ref_intersect(accel, shapes, rays, btn=None, btl=None, kng=None, kn=None):
    shapes = np.ascontiguousarray(shapes)
    rays = np.ascontiguousarray(rays)
    n = len(rays)
    t = np.zeros(n, np.float32)
    ids = np.zeros(n, np.uint32)
    hit = np.zeros(n, np.int32)
    ref().ref_intersect(accel, _ptr(shapes), len(shapes), _ptr(btn), _ptr(btl), _ptr(kng),
                        len(kng) if kng is not None else 0, _ptr(kn),
                        len(kn) if kn is not None else 0, _ptr(rays), n, _ptr(t), _ptr(ids),
                        _ptr(hit))
    return t, ids, hit
