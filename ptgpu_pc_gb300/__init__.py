"""GB300 (sm_103a) LBVH builder and path tracer behind the C ABI of
include/ptgpu.h.

`Context` is a thin ctypes mirror of the C functions: it exists for the tests
and the benchmark; the product is libptgpu.so.  Loading fails loudly when the
library has not been built -- there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("PTGPU_LIB", os.path.join(HERE, "libptgpu.so"))

# every entry point declared in include/ptgpu.h
EXPORTS = [
    "ptgpu_create", "ptgpu_destroy", "ptgpu_status_string", "ptgpu_last_error",
    "ptgpu_abi_version", "ptgpu_read_scene", "ptgpu_stream_scene", "ptgpu_set_shapes", "ptgpu_get_shape_count",
    "ptgpu_get_shapes", "ptgpu_update_camera", "ptgpu_set_camera", "ptgpu_get_camera",
    "ptgpu_build", "ptgpu_get_bvh", "ptgpu_get_kdtree", "ptgpu_get_kdtree_wide", "ptgpu_set_bvh", "ptgpu_last_build_ms", "ptgpu_set_wait_limit",
    "ptgpu_make_seeds", "ptgpu_set_seeds", "ptgpu_get_seeds", "ptgpu_reset_accumulation",
    "ptgpu_draw_frame", "ptgpu_render_async", "ptgpu_synchronize", "ptgpu_get_colors",
    "ptgpu_get_pixels", "ptgpu_get_current_sample", "ptgpu_trace_closest",
    "ptgpu_trace_closest_device", "ptgpu_trace_closest_stats", "ptgpu_get_stream", "ptgpu_render_stats",
    "ptgpu_build_bvh_noalloc",
    "ptgpu_batch_create", "ptgpu_batch_destroy", "ptgpu_batch_add", "ptgpu_batch_build",
    "ptgpu_batch_tune", "ptgpu_batch_render", "ptgpu_batch_reset", "ptgpu_batch_get_pixels",
    "ptgpu_batch_get_colors", "ptgpu_batch_get_bvh", "ptgpu_batch_info_get",
    "ptgpu_server_create", "ptgpu_server_destroy", "ptgpu_server_add_scene", "ptgpu_server_add_scene_file",
    "ptgpu_server_submit",
    "ptgpu_server_wait", "ptgpu_server_info_get", "ptgpu_server_cancel", "ptgpu_server_preview",
    "ptgpu_encode_image", "ptgpu_write_image",
]

_lib = None


class PtgpuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%d): %s" % (_status_name(status), status, msg))
        self.status = status


def _status_name(s):
    return {0: "ok", -1: "E_INVAL", -2: "E_OOM", -3: "E_DEVICE", -4: "E_TIMEOUT",
            -5: "E_IO", -6: "E_RANGE", -7: "E_STATE", -8: "E_CANCELED"}.get(s, "E_?")


def lib():
    """Loads libptgpu.so (raises if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libptgpu.so is not built; run __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, u32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32
        for name in EXPORTS:
            getattr(L, name).restype = ctypes.c_int
        L.ptgpu_status_string.restype = ctypes.c_char_p
        L.ptgpu_last_error.restype = ctypes.c_char_p
        L.ptgpu_create.argtypes = [vp, ctypes.POINTER(vp)]
        L.ptgpu_destroy.argtypes = [vp]
        L.ptgpu_read_scene.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(i32)]
        L.ptgpu_stream_scene.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(i32)]
        L.ptgpu_set_shapes.argtypes = [vp, vp, u32, u32]
        L.ptgpu_get_shape_count.argtypes = [vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
        L.ptgpu_get_shapes.argtypes = [vp, vp, u32]
        L.ptgpu_update_camera.argtypes = [vp]
        L.ptgpu_set_camera.argtypes = [vp, vp]
        L.ptgpu_get_camera.argtypes = [vp, vp]
        L.ptgpu_build.argtypes = [vp, i32, u32]
        L.ptgpu_build_bvh_noalloc.argtypes = [vp, u32, vp, vp, vp]
        L.ptgpu_batch_create.argtypes = [i32, u32, ctypes.POINTER(vp)]
        L.ptgpu_batch_destroy.argtypes = [vp]
        L.ptgpu_batch_add.argtypes = [vp, vp, ctypes.POINTER(i32)]
        L.ptgpu_batch_build.argtypes = [vp, u32]
        L.ptgpu_batch_tune.argtypes = [vp]
        L.ptgpu_batch_render.argtypes = [vp]
        L.ptgpu_batch_reset.argtypes = [vp]
        L.ptgpu_batch_get_pixels.argtypes = [vp, i32, vp]
        L.ptgpu_batch_get_colors.argtypes = [vp, i32, vp]
        L.ptgpu_batch_get_bvh.argtypes = [vp, i32, vp, vp]
        L.ptgpu_batch_info_get.argtypes = [vp, vp]
        L.ptgpu_server_create.argtypes = [i32, ctypes.c_int64, i32, u32, ctypes.POINTER(vp)]
        L.ptgpu_server_destroy.argtypes = [vp]
        L.ptgpu_server_add_scene.argtypes = [vp, vp, u32, u32, u32, ctypes.POINTER(i32)]
        L.ptgpu_server_add_scene_file.argtypes = [vp, ctypes.c_char_p, u32, ctypes.POINTER(i32)]
        L.ptgpu_server_submit.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_int64)]
        L.ptgpu_server_wait.argtypes = [vp, ctypes.c_int64, vp, vp, vp]
        L.ptgpu_server_info_get.argtypes = [vp, vp]
        L.ptgpu_server_cancel.argtypes = [vp, ctypes.c_int64]
        L.ptgpu_server_preview.argtypes = [vp, ctypes.c_int64, vp, vp, ctypes.POINTER(i32)]
        L.ptgpu_get_bvh.argtypes = [vp, vp, vp]
        L.ptgpu_set_bvh.argtypes = [vp, vp, vp, u32]
        L.ptgpu_get_kdtree.argtypes = [vp, vp, ctypes.POINTER(i32), vp, ctypes.POINTER(i32)]
        L.ptgpu_get_kdtree_wide.argtypes = [vp, vp, ctypes.POINTER(i32), vp, ctypes.POINTER(i32)]
        L.ptgpu_last_build_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_float)]
        L.ptgpu_set_wait_limit.argtypes = [vp, u32]
        L.ptgpu_encode_image.argtypes = [vp, i32, vp, ctypes.POINTER(ctypes.c_uint64)]
        L.ptgpu_write_image.argtypes = [vp, ctypes.c_char_p, i32]
        L.ptgpu_make_seeds.argtypes = [ctypes.c_uint64, vp, u32]
        L.ptgpu_set_seeds.argtypes = [vp, vp]
        L.ptgpu_get_seeds.argtypes = [vp, vp]
        L.ptgpu_reset_accumulation.argtypes = [vp]
        L.ptgpu_draw_frame.argtypes = [vp, u32, ctypes.POINTER(vp)]
        L.ptgpu_render_async.argtypes = [vp, u32]
        L.ptgpu_synchronize.argtypes = [vp]
        L.ptgpu_get_colors.argtypes = [vp, vp]
        L.ptgpu_get_pixels.argtypes = [vp, vp]
        L.ptgpu_get_current_sample.argtypes = [vp, ctypes.POINTER(i32)]
        L.ptgpu_trace_closest.argtypes = [vp, vp, u32, vp, vp, vp]
        L.ptgpu_trace_closest_device.argtypes = [vp, vp, u32, vp, vp, vp]
        L.ptgpu_trace_closest_stats.argtypes = [vp, vp, u32, vp, vp, vp, vp]
        L.ptgpu_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
        L.ptgpu_render_stats.argtypes = [vp, u32, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(st):
    if st != 0:
        raise PtgpuError(st, lib().ptgpu_last_error().decode(errors="replace"))


def make_seeds(master, count):
    s = np.zeros(count, np.uint32)
    _check(lib().ptgpu_make_seeds(master, _p(s), count))
    return s


def update_camera(cam):
    c = np.array(cam, abi.CAMERA).reshape(1)
    _check(lib().ptgpu_update_camera(_p(c)))
    return c[0]


class Context:
    """One ptgpu_ctx: a scene, its acceleration structure and a frame."""

    def __init__(self, width, height, accel=abi.ACCEL_BVH, max_depth=0, device=0,
                 block_size=0, flags=0, stream=None, rr_depth=0):
        cfg = np.zeros(1, abi.CONFIG)
        cfg["device"], cfg["accel"], cfg["max_depth"] = device, accel, max_depth
        cfg["width"], cfg["height"] = width, height
        cfg["block_size"], cfg["flags"] = block_size, flags
        cfg["rr_depth"] = rr_depth
        cfg["stream"] = int(stream or 0)
        self._h = ctypes.c_void_p()
        self.width, self.height = width, height
        _check(lib().ptgpu_create(_p(cfg), ctypes.byref(self._h)))
        self.n = 0

    def close(self):
        if self._h:
            lib().ptgpu_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def read_scene(self, path):
        wl = ctypes.c_int32()
        _check(lib().ptgpu_read_scene(self._h, path.encode(), ctypes.byref(wl)))
        n, lc = ctypes.c_uint32(), ctypes.c_uint32()
        _check(lib().ptgpu_get_shape_count(self._h, ctypes.byref(n), ctypes.byref(lc)))
        self.n = n.value
        return wl.value

    def stream_scene(self, path):
        """read_scene without a host copy of the shapes: models are read on
        host threads and expanded into shapes on the device."""
        wl = ctypes.c_int32()
        _check(lib().ptgpu_stream_scene(self._h, path.encode(), ctypes.byref(wl)))
        n, lc = ctypes.c_uint32(), ctypes.c_uint32()
        _check(lib().ptgpu_get_shape_count(self._h, ctypes.byref(n), ctypes.byref(lc)))
        self.n = n.value
        return wl.value

    def set_shapes(self, shapes, light_cnt):
        shapes = abi.as_struct(shapes, abi.SHAPE)
        _check(lib().ptgpu_set_shapes(self._h, _p(shapes), len(shapes), light_cnt))
        self.n = len(shapes)

    def shape_count(self):
        n, lc = ctypes.c_uint32(), ctypes.c_uint32()
        _check(lib().ptgpu_get_shape_count(self._h, ctypes.byref(n), ctypes.byref(lc)))
        return n.value, lc.value

    def get_shapes(self):
        out = np.zeros(self.n, abi.SHAPE)
        _check(lib().ptgpu_get_shapes(self._h, _p(out), self.n))
        return out

    def set_camera(self, cam):
        c = np.array(cam, abi.CAMERA).reshape(1)
        _check(lib().ptgpu_set_camera(self._h, _p(c)))

    def get_camera(self):
        c = np.zeros(1, abi.CAMERA)
        _check(lib().ptgpu_get_camera(self._h, _p(c)))
        return c[0]

    def build(self, accel=abi.ACCEL_BVH, flags=0):
        _check(lib().ptgpu_build(self._h, accel, flags))

    def encode_image(self, fmt=0):
        """The frame as image file bytes (abi.IMAGE_PPM: the reference's P3
        dump; abi.IMAGE_PFM: the float running mean)."""
        n = ctypes.c_uint64()
        _check(lib().ptgpu_encode_image(self._h, fmt, None, ctypes.byref(n)))
        buf = np.zeros(n.value, np.uint8)
        _check(lib().ptgpu_encode_image(self._h, fmt, _p(buf), ctypes.byref(n)))
        return buf.tobytes()

    def write_image(self, path, fmt=0):
        _check(lib().ptgpu_write_image(self._h, str(path).encode(), fmt))

    def set_wait_limit(self, polls):
        """Look-back polls before a build gives up with E_TIMEOUT (0: at the
        first wait; abi.WAIT_LIMIT_DEFAULT restores the default)."""
        _check(lib().ptgpu_set_wait_limit(self._h, int(polls)))

    def last_build_ms(self):
        ms = ctypes.c_float()
        _check(lib().ptgpu_last_build_ms(self._h, ctypes.byref(ms)))
        return ms.value

    def get_bvh(self):
        btn = np.zeros(max(self.n - 1, 1), abi.BVH_NODE)
        btl = np.zeros(self.n, abi.BVH_NODE)
        _check(lib().ptgpu_get_bvh(self._h, _p(btn), _p(btl)))
        return btn[: max(self.n - 1, 0)], btl

    def set_bvh(self, btn, btl):
        btn = abi.as_struct(btn if len(btn) else np.zeros(1, abi.BVH_NODE), abi.BVH_NODE)
        btl = abi.as_struct(btl, abi.BVH_NODE)
        _check(lib().ptgpu_set_bvh(self._h, _p(btn), _p(btl), len(btl)))

    def get_kdtree(self):
        """Returns (kng, kn) or raises PtgpuError(E_RANGE) if it does not fit."""
        kc, nc = ctypes.c_int32(), ctypes.c_int32()
        _check(lib().ptgpu_get_kdtree(self._h, None, ctypes.byref(kc), None, ctypes.byref(nc)))
        kng = np.zeros(kc.value, abi.KD_NODE)
        kn = np.zeros(max(nc.value, 1), np.int32)
        _check(lib().ptgpu_get_kdtree(self._h, _p(kng), ctypes.byref(kc), _p(kn), ctypes.byref(nc)))
        return kng, kn[: nc.value]

    def get_kdtree_wide(self):
        """Returns (nodes, kn): the KD tree breadth-first with 32-bit fields."""
        kc, nc = ctypes.c_int32(), ctypes.c_int32()
        _check(lib().ptgpu_get_kdtree_wide(self._h, None, ctypes.byref(kc), None, ctypes.byref(nc)))
        nodes = np.zeros(max(kc.value, 1), abi.KD_NODE_WIDE)
        kn = np.zeros(max(nc.value, 1), np.int32)
        _check(lib().ptgpu_get_kdtree_wide(self._h, _p(nodes), ctypes.byref(kc), _p(kn), ctypes.byref(nc)))
        return nodes[: kc.value], kn[: nc.value]

    def set_seeds(self, seeds):
        seeds = np.ascontiguousarray(seeds, np.uint32)
        assert seeds.size == 2 * self.width * self.height
        _check(lib().ptgpu_set_seeds(self._h, _p(seeds)))

    def get_seeds(self):
        s = np.zeros(2 * self.width * self.height, np.uint32)
        _check(lib().ptgpu_get_seeds(self._h, _p(s)))
        return s

    def reset(self):
        _check(lib().ptgpu_reset_accumulation(self._h))

    def draw_frame(self, passes):
        """DrawFrame: returns a copy of the RGBA8 pixels."""
        ptr = ctypes.c_void_p()
        _check(lib().ptgpu_draw_frame(self._h, passes, ctypes.byref(ptr)))
        buf = (ctypes.c_uint32 * (self.width * self.height)).from_address(ptr.value)
        return np.frombuffer(buf, np.uint32).copy()

    def draw_frame_view(self, passes):
        """DrawFrame without copying: a view of the library-owned pixels."""
        ptr = ctypes.c_void_p()
        _check(lib().ptgpu_draw_frame(self._h, passes, ctypes.byref(ptr)))
        buf = (ctypes.c_uint32 * (self.width * self.height)).from_address(ptr.value)
        return np.frombuffer(buf, np.uint32)

    def render_async(self, passes):
        _check(lib().ptgpu_render_async(self._h, passes))

    def render_stats(self, passes):
        st = np.zeros(6, np.uint64)
        _check(lib().ptgpu_render_stats(self._h, passes, _p(st)))
        return st

    def synchronize(self):
        _check(lib().ptgpu_synchronize(self._h))

    def get_colors(self):
        c = np.zeros(self.width * self.height, abi.VEC)
        _check(lib().ptgpu_get_colors(self._h, _p(c)))
        return c

    def get_pixels(self):
        p = np.zeros(self.width * self.height, np.uint32)
        _check(lib().ptgpu_get_pixels(self._h, _p(p)))
        return p

    def current_sample(self):
        cs = ctypes.c_int32()
        _check(lib().ptgpu_get_current_sample(self._h, ctypes.byref(cs)))
        return cs.value

    def trace_closest(self, rays):
        rays = abi.as_struct(rays, abi.RAY)
        n = len(rays)
        t = np.zeros(n, np.float32)
        ids = np.zeros(n, np.uint32)
        hit = np.zeros(n, np.int32)
        _check(lib().ptgpu_trace_closest(self._h, _p(rays), n, _p(t), _p(ids), _p(hit)))
        return t, ids, hit

    def trace_closest_device(self, d_rays, n, d_t, d_id, d_hit):
        _check(lib().ptgpu_trace_closest_device(self._h, ctypes.c_void_p(d_rays), n,
                                                ctypes.c_void_p(d_t), ctypes.c_void_p(d_id),
                                                ctypes.c_void_p(d_hit)))

    def trace_closest_stats_device(self, d_rays, n, d_t, d_id, d_hit):
        """trace_closest_device with counters: (node visits, primitive tests)."""
        st = np.zeros(2, np.uint64)
        _check(lib().ptgpu_trace_closest_stats(self._h, ctypes.c_void_p(d_rays), n, ctypes.c_void_p(d_t),
                                               ctypes.c_void_p(d_id), ctypes.c_void_p(d_hit), _p(st)))
        return int(st[0]), int(st[1])

    def stream(self):
        s = ctypes.c_void_p()
        _check(lib().ptgpu_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0


class Batch:
    """Many scenes, one segmented LBVH build and one graph-replayed render
    launch (ptgpu_batch_* in include/ptgpu.h)."""

    def __init__(self, device=0, flags=0):
        self._h = ctypes.c_void_p()
        _check(lib().ptgpu_batch_create(device, flags, ctypes.byref(self._h)))
        self._scenes = []

    def add(self, shapes, light_cnt, camera, width, height, passes, seeds, max_depth=0):
        """Adds a scene (copied); returns its id."""
        shapes = abi.as_struct(shapes, abi.SHAPE)
        seeds = np.ascontiguousarray(seeds, np.uint32)
        if seeds.size != 2 * width * height:
            raise ValueError("seeds must hold 2*width*height words")
        d = np.zeros(1, abi.SCENE)
        d["shapes"] = shapes.ctypes.data
        d["n"], d["light_cnt"] = len(shapes), light_cnt
        d["camera"] = np.array(camera, abi.CAMERA)
        d["width"], d["height"], d["passes"], d["max_depth"] = width, height, passes, max_depth
        d["seeds"] = seeds.ctypes.data
        sid = ctypes.c_int32()
        _check(lib().ptgpu_batch_add(self._h, d.ctypes.data, ctypes.byref(sid)))
        self._scenes.append((width, height, len(shapes)))
        return sid.value

    def build(self, flags=0):
        _check(lib().ptgpu_batch_build(self._h, flags))

    def tune(self):
        _check(lib().ptgpu_batch_tune(self._h))

    def render(self):
        _check(lib().ptgpu_batch_render(self._h))

    def reset(self):
        _check(lib().ptgpu_batch_reset(self._h))

    def pixels(self, scene):
        w, h, _ = self._scenes[scene]
        out = np.zeros(w * h, np.uint32)
        _check(lib().ptgpu_batch_get_pixels(self._h, scene, out.ctypes.data))
        return out

    def colors(self, scene):
        w, h, _ = self._scenes[scene]
        out = np.zeros((w * h, 3), np.float32)
        _check(lib().ptgpu_batch_get_colors(self._h, scene, out.ctypes.data))
        return out

    def bvh(self, scene):
        n = self._scenes[scene][2]
        btn = np.zeros(n - 1, abi.BVH_NODE)
        btl = np.zeros(n, abi.BVH_NODE)
        _check(lib().ptgpu_batch_get_bvh(self._h, scene, btn.ctypes.data, btl.ctypes.data))
        return btn, btl

    def info(self):
        out = np.zeros(1, abi.BATCH_INFO)
        _check(lib().ptgpu_batch_info_get(self._h, out.ctypes.data))
        return {k: out[k][0].item() for k in abi.BATCH_INFO.names}

    def close(self):
        if self._h:
            lib().ptgpu_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Render serving with continuous batching (ptgpu_server_* in
    include/ptgpu.h): scenes registered once, built on first use and kept
    resident under LRU within an HBM budget; submit() and wait() may be
    called from any thread."""

    def __init__(self, device=0, budget_bytes=120 << 30, quantum=0, flags=0):
        self._h = ctypes.c_void_p()
        _check(lib().ptgpu_server_create(device, budget_bytes, quantum, flags, ctypes.byref(self._h)))
        self._sizes = {}

    def add_scene(self, shapes, light_cnt, build_flags=0):
        shapes = abi.as_struct(shapes, abi.SHAPE)
        sid = ctypes.c_int32()
        _check(lib().ptgpu_server_add_scene(self._h, shapes.ctypes.data, len(shapes), light_cnt,
                                            build_flags, ctypes.byref(sid)))
        return sid.value

    def add_scene_file(self, path, build_flags=0):
        """A scene by its file, read again (models expanded on the device)
        whenever it has to be built."""
        sid = ctypes.c_int32()
        _check(lib().ptgpu_server_add_scene_file(self._h, path.encode(), build_flags, ctypes.byref(sid)))
        return sid.value

    def submit(self, scene, camera, width, height, spp, seed, max_depth=0):
        r = np.zeros(1, abi.REQUEST)
        r["scene"], r["width"], r["height"], r["spp"] = scene, width, height, spp
        r["max_depth"], r["seed"] = max_depth, seed
        r["camera"] = np.array(camera, abi.CAMERA)
        t = ctypes.c_int64()
        _check(lib().ptgpu_server_submit(self._h, r.ctypes.data, ctypes.byref(t)))
        self._sizes[t.value] = (width, height)
        return t.value

    def wait(self, ticket, want_pixels=True, want_colors=True):
        """Blocks until the request is done: (pixels, colours, stats)."""
        w, h = self._sizes.pop(ticket)
        px = np.zeros(w * h, np.uint32) if want_pixels else None
        col = np.zeros((w * h, 3), np.float32) if want_colors else None
        st = np.zeros(1, abi.REQUEST_STATS)
        _check(lib().ptgpu_server_wait(self._h, ticket, px.ctypes.data if px is not None else None,
                                       col.ctypes.data if col is not None else None, st.ctypes.data))
        return px, col, {k: st[k][0].item() for k in abi.REQUEST_STATS.names}

    def cancel(self, ticket):
        """Cancels a request; its wait() then raises E_CANCELED."""
        _check(lib().ptgpu_server_cancel(self._h, ctypes.c_int64(ticket)))

    def preview(self, ticket, want_pixels=True, want_colors=True):
        """The request's image after its last finished step: (pixels,
        colours, passes)."""
        w, h = self._sizes[ticket]
        px = np.zeros(w * h, np.uint32) if want_pixels else None
        col = np.zeros((w * h, 3), np.float32) if want_colors else None
        n = ctypes.c_int32()
        _check(lib().ptgpu_server_preview(self._h, ctypes.c_int64(ticket),
                                          px.ctypes.data if px is not None else None,
                                          col.ctypes.data if col is not None else None, ctypes.byref(n)))
        return px, col, n.value

    def info(self):
        out = np.zeros(1, abi.SERVER_INFO)
        _check(lib().ptgpu_server_info_get(self._h, out.ctypes.data))
        return {k: out[k][0].item() for k in abi.SERVER_INFO.names}

    def close(self):
        if self._h:
            lib().ptgpu_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
