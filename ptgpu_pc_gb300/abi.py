"""numpy views of the C-ABI structs declared in include/ptgpu.h.

Each dtype keeps the byte layout of the reference struct it mirrors
(include/geom.h:48-91, camera.h:29-38, BVHNodeGPU.h:4-16, KDNodeGPU.h:4-14),
so arrays built here can be handed to the C ABI, the oracle or the
reference's own code unchanged.
"""
import numpy as np

SPHERE, TRIANGLE = 0, 1
DIFF, SPEC, REFR = 0, 1, 2
ACCEL_NONE, ACCEL_BVH, ACCEL_KDTREE = 0, 1, 2
WAIT_LIMIT_DEFAULT = 4194304      # PTGPU_WAIT_LIMIT_DEFAULT
IMAGE_PPM, IMAGE_PFM = 0, 1       # PTGPU_IMAGE_*

VEC = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4")])
RAY = np.dtype({"names": ["o", "d"], "formats": [("<f4", 3), ("<f4", 3)],
                "offsets": [0, 12], "itemsize": 24})
BOUND = np.dtype(("<f4", 6))  # min_x, max_x, min_y, max_y, min_z, max_z

SHAPE = np.dtype({
    "names": ["type", "p1", "p2", "p3", "rad", "center", "e", "c", "refl",
              "index", "morton_code", "b", "area"],
    "formats": ["<i4", ("<f4", 3), ("<f4", 3), ("<f4", 3), "<f4", ("<f4", 3),
                ("<f4", 3), ("<f4", 3), "<i4", "<i4", "<u4", ("<f4", 6), "<f4"],
    "offsets": [0, 4, 16, 28, 4, 8, 40, 52, 64, 68, 72, 76, 100],
    "itemsize": 104,
})

CAMERA = np.dtype({
    "names": ["orig", "target", "pitch", "yaw", "width", "height", "dir", "x", "y"],
    "formats": [("<f4", 3), ("<f4", 3), "<f4", "<f4", "<f4", "<f4", ("<f4", 3),
                ("<f4", 3), ("<f4", 3)],
    "offsets": [0, 12, 24, 28, 32, 36, 40, 52, 64],
    "itemsize": 76,
})

BVH_NODE = np.dtype({
    "names": ["min", "max", "nShape", "leaf", "nLeft", "nRight", "nParent",
              "bound", "cost", "area"],
    "formats": ["<i4"] * 7 + [("<f4", 6), "<f4", "<f4"],
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 52, 56],
    "itemsize": 60,
})

KD_NODE = np.dtype({
    "names": ["leaf", "nLeft", "nRight", "nParent", "bound", "min", "max"],
    "formats": ["<i2"] * 4 + [("<f4", 6), "<i2", "<i2"],
    "offsets": [0, 2, 4, 6, 8, 32, 34],
    "itemsize": 36,
})

KD_NODE_WIDE = np.dtype({
    "names": ["leaf", "nLeft", "nRight", "nParent", "bound", "min", "max"],
    "formats": ["<i4"] * 4 + [("<f4", 6), "<i4", "<i4"],
    "offsets": [0, 4, 8, 12, 16, 40, 44],
    "itemsize": 48,
})

CONFIG = np.dtype({
    "names": ["device", "accel", "max_depth", "width", "height", "block_size",
              "flags", "rr_depth", "stream"],
    "formats": ["<i4"] * 8 + ["<u8"],
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32],
    "itemsize": 40,
})

# ptgpu_scene / ptgpu_batch_info (batched renders)
SCENE = np.dtype({
    "names": ["shapes", "n", "light_cnt", "camera", "width", "height", "passes", "max_depth",
              "seeds"],
    "formats": ["<u8", "<u4", "<u4", CAMERA, "<i4", "<i4", "<i4", "<i4", "<u8"],
    "offsets": [0, 8, 12, 16, 92, 96, 100, 104, 112],
    "itemsize": 120,
})

BATCH_INFO = np.dtype({
    "names": ["build_ms", "render_ms", "samples", "block", "refill", "stack", "tree_depth",
              "shapes"],
    "formats": ["<f4", "<f4", "<f8", "<i4", "<i4", "<i4", "<i4", "<i8"],
    "offsets": [0, 4, 8, 16, 20, 24, 28, 32],
    "itemsize": 40,
})

# ptgpu_request / ptgpu_request_stats / ptgpu_server_info (serving)
REQUEST = np.dtype({
    "names": ["scene", "width", "height", "spp", "max_depth", "pad", "seed", "camera"],
    "formats": ["<i4"] * 6 + ["<u8", CAMERA],
    "offsets": [0, 4, 8, 12, 16, 20, 24, 32],
    "itemsize": 112,
})

REQUEST_STATS = np.dtype({
    "names": ["queued_ms", "latency_ms", "steps", "built"],
    "formats": ["<f8", "<f8", "<i4", "<i4"],
    "offsets": [0, 8, 16, 20],
    "itemsize": 24,
})

SERVER_INFO = np.dtype({
    "names": ["budget_bytes", "bytes_in_use", "requests_done", "builds", "evictions", "steps",
              "resident_scenes", "active_requests", "pending_requests", "quantum", "samples_done",
              "shape_slots_used", "pixel_slots_used", "light_slots_used"],
    "formats": ["<i8"] * 6 + ["<i4"] * 4 + ["<f8"] + ["<i8"] * 3,
    "offsets": [0, 8, 16, 24, 32, 40, 48, 52, 56, 60, 64, 72, 80, 88],
    "itemsize": 96,
})

# status codes (include/ptgpu.h)
OK, E_INVAL, E_OOM, E_DEVICE, E_TIMEOUT, E_IO, E_RANGE, E_STATE = 0, -1, -2, -3, -4, -5, -6, -7
E_CANCELED = -8

FLAG_WAVEFRONT = 0x1
FLAG_MORTON_DELTA = 0x2        # reserved: ptgpu_build answers E_INVAL
FLAG_TREELET = 0x4
FLAG_ARGS_RTL = 0x8
SERVER_ALL_ACTIVE = 0x100
FLAG_WIDE_TRAVERSAL = 0x10
FLAG_KD_HOST = 0x20
FLAG_ROW_ORDER = 0x40


def treelet_sweeps(n):
    """Build flag field: rounds of the treelet stage (0 or 1 = one round)."""
    return (n & 0xF) << 8


def triangles(p1, p2, p3, e=(0.0, 0.0, 0.0), c=(0.75, 0.75, 0.75), refl=DIFF):
    """Shape array of triangles with per-shape or shared emission/colour."""
    p1 = np.asarray(p1, np.float32).reshape(-1, 3)
    n = p1.shape[0]
    s = np.zeros(n, SHAPE)
    s["type"] = TRIANGLE
    s["p1"], s["p2"], s["p3"] = p1, np.asarray(p2, np.float32), np.asarray(p3, np.float32)
    s["e"], s["c"], s["refl"] = e, c, refl
    e1 = s["p2"] - s["p1"]
    e2 = s["p3"] - s["p1"]
    s["area"] = tri_area(e1, e2)
    return s


def tri_area(e1, e2):
    """norm(cross(e1, e2)) * 0.5f in float32, as ReadTxt computes it
    (displayfunc.cpp:315-318)."""
    e1 = e1.astype(np.float32)
    e2 = e2.astype(np.float32)
    nx = e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1]
    ny = e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2]
    nz = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
    return (np.sqrt(nx * nx + ny * ny + nz * nz) * np.float32(0.5)).astype(np.float32)


def spheres(rad, center, e, c, refl):
    rad = np.asarray(rad, np.float32).reshape(-1)
    n = rad.shape[0]
    s = np.zeros(n, SHAPE)
    s["type"] = SPHERE
    s["rad"] = rad
    s["center"] = np.asarray(center, np.float32).reshape(n, 3)
    s["e"] = np.asarray(e, np.float32).reshape(n, 3)
    s["c"] = np.asarray(c, np.float32).reshape(n, 3)
    s["refl"] = np.asarray(refl).reshape(n)
    # area = 4 * FLOAT_PI * r * r (displayfunc.cpp:282), left to right in float32
    s["area"] = (np.float32(4.0) * np.float32(3.14159265358979323846) * rad) * rad
    return s


def light_count(shapes):
    e = shapes["e"]
    return int(np.count_nonzero(np.any(e != 0, axis=1)))


def concat_shapes(*arrays):
    """Concatenates Shape arrays keeping the 104-byte layout (np.concatenate
    would repack the overlapping union fields)."""
    raw = [np.ascontiguousarray(a).view(np.uint8).reshape(len(a), SHAPE.itemsize) for a in arrays]
    return np.ascontiguousarray(np.concatenate(raw, axis=0)).view(SHAPE).reshape(-1)


def as_struct(a, dtype):
    """Checks that `a` has exactly the ABI dtype and is contiguous."""
    a = np.ascontiguousarray(a)
    if a.dtype != dtype or a.dtype.itemsize != dtype.itemsize:
        raise TypeError("expected dtype %r with itemsize %d, got %r" % (dtype, dtype.itemsize, a.dtype))
    return a
