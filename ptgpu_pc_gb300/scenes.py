"""Seeded synthetic scenes and ray sets for the benchmark workloads.

These stand in for the reference's interactive scenes: the reference has no
benchmark suite, so every workload is generated here from a fixed seed, and
the same arrays feed the GPU library, the oracle and the reference's own code.

  cornell_spheres()      9-sphere Cornell box, 256x256, 16 spp, depth 6
  icosphere_scene()      displaced level-6 icosphere + 12 wall triangles +
                         2-triangle area light (81,934 shapes), 512x512
  triangle_soup(n)       n random triangles in the unit cube (1M / 4M)
  random_rays(n)         seeded rays, origins in [-0.5,1.5]^3, uniform dirs
  batch_scenes()         64 mixed scenes (triangle counts log-uniform)
"""
import functools
import math

import numpy as np

from . import abi

F32 = np.float32


def camera(orig, pitch=0.0, yaw=0.0, target=None, width=0, height=0):
    c = np.zeros(1, abi.CAMERA)[0]
    c["orig"] = orig
    c["target"] = target if target is not None else orig
    c["pitch"], c["yaw"] = pitch, yaw
    c["width"], c["height"] = width, height
    return c


# ---------------------------------------------------------------------------
# Cornell box of spheres (smallpt layout)
# ---------------------------------------------------------------------------
def cornell_spheres():
    """Returns (shapes, light_cnt, camera).  Walls are r=1e5 spheres bounding
    x in [1,99], y in [0,81.6], z in [0,170]; mirror and glass r=16.5 spheres
    (colour .9 as in include/scene.h:54-55); a r=600 light sphere above the
    ceiling with emission 12.  The camera at (50,52,295.6) looks along
    (0,-0.0427,-1): the reference camera is pitch/yaw only, so the pitch is
    asin(0.0427/|(0,-0.0427,-1)|) and the yaw 0."""
    R = 1e5
    rad = [R, R, R, R, R, R, 16.5, 16.5, 600.0]
    center = [[R + 1, 40.8, 81.6], [-R + 99, 40.8, 81.6], [50, 40.8, R],
              [50, 40.8, -R + 170], [50, R, 81.6], [50, -R + 81.6, 81.6],
              [27, 16.5, 47], [73, 16.5, 78], [50, 681.33, 81.6]]
    e = [[0, 0, 0]] * 8 + [[12, 12, 12]]
    c = [[.75, .25, .25], [.25, .25, .75], [.75, .75, .75], [.75, .75, .75],
         [.75, .75, .75], [.75, .75, .75], [.9, .9, .9], [.9, .9, .9], [0, 0, 0]]
    refl = [abi.DIFF] * 6 + [abi.SPEC, abi.REFR, abi.DIFF]
    shapes = abi.spheres(rad, center, e, c, refl)
    pitch = math.asin(0.0427 / math.sqrt(0.0427 ** 2 + 1.0))
    cam = camera([50, 52, 295.6], pitch=pitch, yaw=0.0,
                 target=[50, 52 - 0.0427, 295.6 - 1.0])
    return shapes, 1, cam


# ---------------------------------------------------------------------------
# Displaced icosphere in a triangle Cornell box
# ---------------------------------------------------------------------------
def _icosahedron():
    p = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0],
                  [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
                  [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    return v, f


def _subdivide(v, f):
    """One loop of 1-to-4 subdivision with shared edge midpoints."""
    edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
    key = np.sort(edges, axis=1)
    # unique edges in (lo, hi) order, through one int64 code per edge
    code = key[:, 0] * np.int64(len(v)) + key[:, 1]
    ucode, inv = np.unique(code, return_inverse=True)
    uniq = np.stack([ucode // len(v), ucode % len(v)], axis=1)
    mid = v[uniq[:, 0]] + v[uniq[:, 1]]
    mid /= np.linalg.norm(mid, axis=1, keepdims=True)
    base = len(v)
    inv = inv.reshape(3, -1) + base
    a, b, c = f[:, 0], f[:, 1], f[:, 2]
    ab, bc, ca = inv[0], inv[1], inv[2]
    nf = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                         np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)], axis=0)
    return np.concatenate([v, mid], axis=0), nf


@functools.lru_cache(maxsize=None)
def _icosphere_cached(level):
    v, f = _icosahedron()
    for _ in range(level):
        v, f = _subdivide(v, f)
    v.flags.writeable = False
    f.flags.writeable = False
    return v, f


def icosphere(level):
    """Unit icosphere after `level` subdivisions (cached, read-only arrays)."""
    return _icosphere_cached(level)


def value_noise3(p, seed, freq):
    """Seeded 3-D value noise in [-1, 1]: hashed lattice values, smoothstep
    trilinear interpolation."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256)
    vals = rng.uniform(-1.0, 1.0, 256)
    q = p * freq
    i0 = np.floor(q).astype(np.int64)
    fr = q - i0
    w = fr * fr * (3.0 - 2.0 * fr)

    def h(ix, iy, iz):
        return vals[perm[(perm[(perm[ix & 255] + iy) & 255] + iz) & 255]]

    out = np.zeros(len(p))
    for dx in (0, 1):
        wx = w[:, 0] if dx else 1.0 - w[:, 0]
        for dy in (0, 1):
            wy = w[:, 1] if dy else 1.0 - w[:, 1]
            for dz in (0, 1):
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out += wx * wy * wz * h(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz)
    return out


def box_walls():
    """12 wall triangles spanning x in [1,99], y in [0,81.6], z in [0,170]."""
    x0, x1, y0, y1, z0, z1 = 1.0, 99.0, 0.0, 81.6, 0.0, 170.0
    quads = [  # (corners, colour)
        ([[x0, y0, z0], [x0, y1, z0], [x0, y1, z1], [x0, y0, z1]], [.75, .25, .25]),  # left
        ([[x1, y0, z0], [x1, y0, z1], [x1, y1, z1], [x1, y1, z0]], [.25, .25, .75]),  # right
        ([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0]], [.75, .75, .75]),  # back
        ([[x0, y0, z1], [x0, y1, z1], [x1, y1, z1], [x1, y0, z1]], [.75, .75, .75]),  # front
        ([[x0, y0, z0], [x0, y0, z1], [x1, y0, z1], [x1, y0, z0]], [.75, .75, .75]),  # floor
        ([[x0, y1, z0], [x1, y1, z0], [x1, y1, z1], [x0, y1, z1]], [.75, .75, .75]),  # ceiling
    ]
    p1, p2, p3, col = [], [], [], []
    for q, c in quads:
        q = np.array(q, np.float64)
        p1 += [q[0], q[0]]
        p2 += [q[1], q[2]]
        p3 += [q[2], q[3]]
        col += [c, c]
    s = abi.triangles(np.array(p1), np.array(p2), np.array(p3))
    s["c"] = np.array(col, np.float32)
    return s


def area_light(center=(50.0, 81.5, 80.0), half=10.0, emission=12.0):
    """2-triangle square light facing down, just under the ceiling."""
    cx, cy, cz = center
    a = [cx - half, cy, cz - half]
    b = [cx + half, cy, cz - half]
    c = [cx + half, cy, cz + half]
    d = [cx - half, cy, cz + half]
    s = abi.triangles(np.array([a, a], float), np.array([b, c], float), np.array([c, d], float),
                      e=(emission, emission, emission), c=(0.0, 0.0, 0.0))
    return s


def displaced_icosphere(level=6, radius=20.0, center=(50.0, 25.0, 80.0), amp=0.05,
                        freq=4.0, seed=2, albedo=0.75, faces=None):
    """The icosphere radially displaced by value noise; `faces` keeps a subset
    of its faces (the displacement of a vertex does not depend on which faces
    are kept)."""
    v, f = icosphere(level)
    if faces is not None:
        f = f[faces]
        used, f = np.unique(f, return_inverse=True)
        f = f.reshape(-1, 3)
        v = v[used]
    n = value_noise3(v, seed, freq)
    r = radius * (1.0 + amp * n)
    pts = v * r[:, None] + np.asarray(center)
    s = abi.triangles(pts[f[:, 0]], pts[f[:, 1]], pts[f[:, 2]], c=(albedo, albedo, albedo))
    return s


def icosphere_scene(level=6, seed=2, n_tris=None):
    """Returns (shapes, light_cnt, camera): the displaced icosphere, the 12
    wall triangles and the 2 light triangles, in that order (the light last,
    where IntersectP does not test it).  n_tris subsamples the icosphere to an
    exact triangle count."""
    n_faces = 20 * 4 ** level
    keep = None
    if n_tris is not None and n_tris < n_faces:
        rng = np.random.default_rng(seed + 1000)
        keep = np.sort(rng.choice(n_faces, n_tris, replace=False))
    ico = displaced_icosphere(level=level, seed=seed, faces=keep)
    shapes = abi.concat_shapes(ico, box_walls(), area_light())
    cam = camera([50.0, 45.0, 168.0], pitch=0.2, yaw=0.0, target=[50.0, 25.0, 80.0])
    return shapes, 2, cam


# ---------------------------------------------------------------------------
# Random triangle soup and ray sets
# ---------------------------------------------------------------------------
def triangle_soup(n, seed=3):
    rng = np.random.default_rng(seed)
    cen = rng.random((n, 3))
    sigma = 0.5 * n ** (-1.0 / 3.0)
    g = rng.normal(0.0, sigma, (n, 3, 3))
    g -= g.mean(axis=1, keepdims=True)
    v = (cen[:, None, :] + g).astype(np.float32)
    s = np.zeros(n, abi.SHAPE)
    s["type"] = abi.TRIANGLE
    s["p1"], s["p2"], s["p3"] = v[:, 0], v[:, 1], v[:, 2]
    s["c"] = (0.75, 0.75, 0.75)
    return s


def random_rays(n, seed=4):
    rng = np.random.default_rng(seed)
    r = np.zeros(n, abi.RAY)
    r["o"] = rng.uniform(-0.5, 1.5, (n, 3)).astype(np.float32)
    u = rng.random(n)
    v = rng.random(n)
    z = 1.0 - 2.0 * u
    rr = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * np.pi * v
    d = np.stack([rr * np.cos(phi), rr * np.sin(phi), z], axis=1)
    r["d"] = d.astype(np.float32)
    return r


# ---------------------------------------------------------------------------
# Mixed batch of scenes (64 scenes from master seed 7)
# ---------------------------------------------------------------------------
RESOLUTIONS = (128, 256, 512, 1024)
SPPS = (1, 4, 16, 64)


def batch_specs(count=64, master_seed=7, tri_min=1000, tri_max=2_000_000):
    """Per-scene (n_tris, level, res, spp, seed) drawn from the master seed."""
    rng = np.random.default_rng(master_seed)
    specs = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(tri_min), math.log(tri_max)))))
        level = max(0, math.ceil(math.log(max(n, 20) / 20.0, 4)))
        res = int(rng.choice(RESOLUTIONS))
        spp = int(rng.choice(SPPS))
        specs.append(dict(n_tris=n, level=level, res=res, spp=spp, seed=int(rng.integers(1 << 30))))
    return specs


def scene_from_spec(spec):
    shapes, lc, cam = icosphere_scene(level=spec["level"], seed=spec["seed"] % 1000,
                                      n_tris=spec["n_tris"])
    return shapes, lc, cam


# ---------------------------------------------------------------------------
# OBJ model and .txt scene files (scene ingestion)
# ---------------------------------------------------------------------------
def write_obj_model(path, n_tris, seed=3, block=64):
    """Writes a seeded OBJ model of about n_tris triangles and returns (path,
    vertices (nv, 3) float32, triangles (nt, 3) int32) as a reader must see
    them.  Vertices come in blocks, each followed by faces on the vertices
    defined so far, in every face form the reader takes: "i", "i/j", "i//k",
    "i/j/k", negative (relative) indices and quads (fanned into two
    triangles); plus comments, vt / vn lines, leading blanks, CRLF and lone
    CR line ends.  Values are written with 9 significant digits, which read
    back to the same float32."""
    rng = np.random.default_rng(seed)
    out, verts, tris = [], [], []
    nv = 0
    ends = ("\n", "\n", "\n", "\r\n", "\r")
    n_faces = 2 * block
    while sum(len(t) for t in tris) < n_tris:
        v = (rng.random((block, 3)) * 100.0 - 50.0).astype(np.float32)
        lead = rng.random(block) < 0.05
        vend = rng.integers(len(ends), size=block)
        for x, ld, en in zip(v.tolist(), lead, vend):
            out.append("%sv %.9g %.9g %.9g%s" % (" " if ld else "", x[0], x[1], x[2], ends[en]))
        verts.append(v)
        nv += block
        if rng.random() < 0.3:
            out.append("# block %d\nvt 0.5 0.5\nvn 0 0 1\n" % nv)
        # distinct corners: a start and up to three steps below nv/4, mod nv
        k = np.where(rng.random(n_faces) < 0.2, 4, 3)
        steps = rng.integers(1, max(2, nv // 4), (n_faces, 3))
        start = rng.integers(0, nv, n_faces)
        idx = np.concatenate([start[:, None], start[:, None] + np.cumsum(steps, axis=1)], axis=1) % nv
        forms = rng.integers(5, size=n_faces)
        fend = rng.integers(len(ends), size=n_faces)
        for q, kk, form, en in zip(idx.tolist(), k.tolist(), forms.tolist(), fend.tolist()):
            q = q[:kk]
            if form == 0:
                toks = ["%d" % (i + 1) for i in q]
            elif form == 1:
                toks = ["%d/1" % (i + 1) for i in q]
            elif form == 2:
                toks = ["%d//1" % (i + 1) for i in q]
            elif form == 3:
                toks = ["%d/1/1" % (i + 1) for i in q]
            else:
                toks = ["%d" % (i - nv) for i in q]     # relative: -1 is the last vertex
            out.append("f " + " ".join(toks) + ends[en])
        tri = np.stack([idx[:, 0], idx[:, 1], idx[:, 2]], axis=1)
        quad = np.stack([idx[k == 4, 0], idx[k == 4, 2], idx[k == 4, 3]], axis=1)
        # fanned triangles in file order: each face's first, then a quad's second
        order = np.concatenate([np.flatnonzero(np.ones(n_faces, bool)) * 2,
                                np.flatnonzero(k == 4) * 2 + 1])
        both = np.concatenate([tri, quad])
        tris.append(both[np.argsort(order, kind="stable")])
    out.append("\n")      # the reader drops the line before the final byte
    with open(path, "w", newline="") as f:
        f.write("".join(out))
    return path, np.concatenate(verts), np.concatenate(tris).astype(np.int32)


def write_model_scene(directory, n_tris, seed=4):
    """A .txt scene (ReadTxt format) mixing spheres, triangle lines and two
    OBJ models of about n_tris/2 triangles each, one of them emitting;
    returns its path."""
    import os
    half = max(1, n_tris // 2)
    m1, _, _ = write_obj_model(os.path.join(str(directory), "m1.obj"), half, seed=seed)
    m2, _, _ = write_obj_model(os.path.join(str(directory), "m2.obj"), half, seed=seed + 1)
    path = os.path.join(str(directory), "scene.txt")
    with open(path, "w") as f:
        f.write("gamma 2.2  sky1 0 0 0  sky2 0 0 0\ncamera 0 10 120  0 0 0\nmaterials 1\n"
                "matte 0.5 0.5 0.5  0.1\nobjects 6\n"
                "sphere 5  0 30 0  4 4 4  0 0 0  0\n"
                "triangle  -60 -50 -60  60 -50 -60  0 -50 60  0 0 0  0.7 0.7 0.7  0\n"
                "model %s  -20 0 0  0.3 0.3 0.3  0 0 0  0.8 0.6 0.4  0\n"
                "sphere 3  20 20 20  0 0 0  0.9 0.9 0.9  2\n"
                "model %s  20 0 0  0.2 0.2 0.2  1.5 1.5 1.5  0.5 0.5 0.5  1\n"
                "triangle  -60 60 -60  60 60 -60  0 60 60  0 0 0  0.7 0.7 0.7  0\n" % (m1, m2))
    return path
