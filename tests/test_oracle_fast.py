"""The oracle's speed-ups for large scenes give the plain oracle's answers.

`make_accel(..., fast=True)` answers shadow queries (IntersectP,
rendering_kernel.cl:375-395: any shape but the last with 0 < d < maxt)
through the tree instead of the brute-force loop, and lets the closest-hit
walk (Intersect, rendering_kernel.cl:194-363) skip boxes that cannot hold a
better hit.  The config-size render tests rely on both, so here they are
compared with the plain forms: shadow answers equal, closest hits equal bit
for bit, renders equal bit for bit."""
import numpy as np
import pytest

from ptgpu_pc_gb300 import abi, scenes


def _accels(orc, shapes, fast):
    _, btn, btl, _ = orc.build_bvh(shapes)
    kd = orc.KD(shapes)
    return {abi.ACCEL_BVH: orc.make_accel(abi.ACCEL_BVH, btn, btl, fast=fast),
            abi.ACCEL_KDTREE: orc.make_accel(abi.ACCEL_KDTREE, kd=kd, fast=fast)}


def _shadow_rays(shapes, n, seed):
    """Segments from points in the box toward the light triangles, toward
    random shape centroids and in random directions."""
    rng = np.random.default_rng(seed)
    o = rng.uniform([1, 0.5, 1], [99, 81, 169], (n, 3)).astype(np.float32)

    def centre(s):
        tri = (s["p1"] + s["p2"] + s["p3"]) / 3
        return np.where((s["type"] == abi.TRIANGLE)[:, None], tri, s["center"]).astype(np.float32)

    k = rng.integers(0, len(shapes), n)
    tgt = centre(shapes[k])
    lights = shapes[(shapes["e"] != 0).any(1)]
    if len(lights):
        j = rng.integers(0, len(lights), n)
        third = np.arange(n) % 3 == 1
        tgt[third] = centre(lights[j])[third]
    rnd = np.arange(n) % 3 == 2
    tgt[rnd] = o[rnd] + rng.normal(size=(rnd.sum(), 3)).astype(np.float32) * 50
    d = tgt - o
    ln = np.sqrt((d * d).sum(1))
    rays = np.zeros(n, abi.RAY)
    rays["o"] = o
    rays["d"] = d / ln[:, None]
    return rays, (ln - 0.01).astype(np.float32)


@pytest.mark.parametrize("scene", ["ico4", "spheres"])
def test_fast_shadow_queries_equal_bruteforce(scene, orc):
    if scene == "ico4":
        shapes, lc, _ = scenes.icosphere_scene(level=4)
    else:
        shapes, lc, _ = scenes.cornell_spheres()
    rays, maxt = _shadow_rays(shapes, 60_000, seed=31)
    brute = orc.shadow_batch(shapes, rays, maxt)
    assert 0.05 < brute.mean() < 0.95
    for accel, acc in _accels(orc, shapes, fast=True).items():
        fast = orc.shadow_batch(shapes, rays, maxt, accel=acc)
        assert np.array_equal(fast, brute), (accel, int((fast != brute).sum()))


def test_fast_shadow_skips_the_last_shape(orc):
    """IntersectP never tests the last shape: a segment blocked only by it
    is unoccluded through the tree as in the loop."""
    shapes = scenes.triangle_soup(2000, seed=32)
    rays = np.zeros(1, abi.RAY)
    last = shapes[-1]
    c = (last["p1"] + last["p2"] + last["p3"]) / 3
    rays["o"] = c + np.array([0, 0, -5], np.float32)
    rays["d"] = np.array([0, 0, 1], np.float32)
    shapes = shapes.copy()
    shapes[:-1]["p1"] += 50; shapes[:-1]["p2"] += 50; shapes[:-1]["p3"] += 50
    maxt = np.array([10.0], np.float32)
    assert orc.shadow_batch(shapes, rays, maxt)[0] == 0
    for acc in _accels(orc, shapes, fast=True).values():
        assert orc.shadow_batch(shapes, rays, maxt, accel=acc)[0] == 0


@pytest.mark.parametrize("accel", [abi.ACCEL_BVH, abi.ACCEL_KDTREE])
def test_culled_closest_hits_equal_plain_walk(accel, orc):
    shapes = scenes.triangle_soup(100_000, seed=33)
    rays = scenes.random_rays(40_000, seed=34)
    plain = orc.trace_closest(shapes, rays, _accels(orc, shapes, False)[accel])
    fast = orc.trace_closest(shapes, rays, _accels(orc, shapes, True)[accel])
    assert np.array_equal(plain[2], fast[2])
    assert np.array_equal(plain[0].view(np.uint32), fast[0].view(np.uint32))
    assert np.array_equal(plain[1], fast[1])


@pytest.mark.parametrize("accel", [abi.ACCEL_BVH, abi.ACCEL_KDTREE])
def test_fast_render_equals_plain_render(accel, orc):
    shapes, lc, cam = scenes.icosphere_scene(level=3)
    w = h = 24
    c = np.array(cam, abi.CAMERA)
    c["width"], c["height"] = w, h
    c = orc.update_camera(c)
    seeds = orc.make_seeds(35, 2 * w * h)
    out = []
    for fast in (False, True):
        col, pix, sd = orc.render(shapes, lc, c, w, h, seeds, 2, accel=_accels(orc, shapes, fast)[accel],
                                  max_depth=8, arg_order_rtl=True)
        out.append((col, pix, sd))
    assert out[0][0].tobytes() == out[1][0].tobytes()
    assert np.array_equal(out[0][2], out[1][2])


def test_oracle_russian_roulette_keeps_the_mean(orc):
    """The opt-in throughput roulette (rr_depth > 0) is unbiased: over 8 seed
    replicas the frame mean with rr_depth = 2 agrees with the plain
    estimator's within 3 combined standard errors, and rr_depth = 0 is the
    plain estimator bit for bit."""
    shapes, lc, cam = scenes.icosphere_scene(level=2)
    w = h = 24
    c = np.array(cam, abi.CAMERA)
    c["width"], c["height"] = w, h
    c = orc.update_camera(c)
    _, btn, btl, _ = orc.build_bvh(shapes)
    acc = orc.make_accel(abi.ACCEL_BVH, btn, btl, fast=True)
    means = {0: [], 2: []}
    for r in range(8):
        seeds = orc.make_seeds(60 + r, 2 * w * h)
        for rr in (0, 2):
            col, _, _ = orc.render(shapes, lc, c, w, h, seeds, 8, accel=acc, max_depth=8, rr_depth=rr)
            means[rr].append(col.view(np.float32).mean())
    a, b = np.array(means[0]), np.array(means[2])
    se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    assert abs(a.mean() - b.mean()) <= 3 * se
    seeds = orc.make_seeds(70, 2 * w * h)
    p0 = orc.render(shapes, lc, c, w, h, seeds, 2, accel=acc, max_depth=8)
    p1 = orc.render(shapes, lc, c, w, h, seeds, 2, accel=acc, max_depth=8, rr_depth=0)
    assert p0[0].tobytes() == p1[0].tobytes()
