"""Fixed, seeded workloads of the hot path for profiling one kernel at a time.

    python -m ptgpu_pc_gb300.cases render  [--width 512 --height 512 --spp 16 --frames 2 --flags 0 --sweeps 2 --accel bvh|kd]
    python -m ptgpu_pc_gb300.cases lbvh    [--n 4194304 --builds 2]
    python -m ptgpu_pc_gb300.cases closest [--n 4194304 --rays 16777216 --reps 2]
    python -m ptgpu_pc_gb300.cases batch   [--scenes 16 --tri-max 200000 --frames 2]
    python -m ptgpu_pc_gb300.cases kd      [--builds 2]
    python -m ptgpu_pc_gb300.cases scene_build [--builds 2 --sweeps 2]
    python -m ptgpu_pc_gb300.cases ingest  [--n 1000000 --reps 2]

render: the displaced-icosphere scene (81,934 shapes) built with `sweeps` treelet rounds,
`frames` frames of `spp` passes each through the lane tracer.  lbvh: builds of
`n` seeded random triangles (the ptgpu_build(ctx, PTGPU_ACCEL_BVH, 0) path).
closest: ptgpu_trace_closest_device on random rays against an LBVH of `n`
random triangles.  batch: a batch of `scenes` mixed icosphere scenes (the
benchmark's spec generator, up to tri-max triangles each), one segmented
build, `frames` batched renders.  kd: GPU KD-tree builds of the benchmark
scene.  ingest: ptgpu_stream_scene of a seeded scene file with two OBJ
models of n triangles in all.  Each case prints one line per repetition with
its device time, so its launch sequence is fixed: set-up launches first, then
the same kernels once per repetition.
"""
import argparse
import time

import numpy as np

import ptgpu_pc_gb300 as pt
from ptgpu_pc_gb300 import abi, scenes


def run_render(a):
    shapes, lc, cam = scenes.icosphere_scene(level=6)
    accel = abi.ACCEL_KDTREE if a.accel == "kd" else abi.ACCEL_BVH
    with pt.Context(a.width, a.height, accel=accel, max_depth=a.max_depth,
                    flags=a.flags) as ctx:
        ctx.set_shapes(shapes, lc)
        if accel == abi.ACCEL_KDTREE:
            ctx.build(abi.ACCEL_KDTREE)
        else:
            ctx.build(abi.ACCEL_BVH, abi.FLAG_TREELET | abi.treelet_sweeps(a.sweeps))
        print("scene build %.3f ms" % ctx.last_build_ms())
        ctx.set_camera(cam)
        ctx.set_seeds(pt.make_seeds(1, 2 * a.width * a.height))
        for i in range(a.frames):
            t0 = time.perf_counter()
            ctx.reset()
            ctx.render_async(a.spp)
            ctx.synchronize()
            print("render %dx%d %d spp frame %d: %.2f ms (host clock)"
                  % (a.width, a.height, a.spp, i, (time.perf_counter() - t0) * 1e3))


def run_scene_build(a):
    shapes, lc, _ = scenes.icosphere_scene(level=6)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, lc)
        for i in range(a.builds):
            ctx.build(abi.ACCEL_BVH, abi.FLAG_TREELET | abi.treelet_sweeps(a.sweeps))
            print("scene build %d (%d treelet rounds): %.3f ms" % (i, a.sweeps, ctx.last_build_ms()))


def run_lbvh(a):
    shapes = scenes.triangle_soup(a.n, seed=3)
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, 0)
        for i in range(a.builds):
            ctx.build(abi.ACCEL_BVH)
            print("lbvh n=%d build %d: %.3f ms" % (a.n, i, ctx.last_build_ms()))


def run_closest(a):
    import torch
    shapes = scenes.triangle_soup(a.n, seed=3)
    rays = scenes.random_rays(a.rays, seed=4)
    d_rays = torch.from_numpy(rays.view(np.uint8).reshape(-1)).cuda()
    d_t = torch.empty(a.rays, dtype=torch.float32, device="cuda")
    d_id = torch.empty(a.rays, dtype=torch.int32, device="cuda")
    d_hit = torch.empty(a.rays, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    with pt.Context(8, 8) as ctx:
        ctx.set_shapes(shapes, 0)
        ctx.build(abi.ACCEL_BVH)
        for i in range(a.reps):
            t0 = time.perf_counter()
            ctx.trace_closest_device(d_rays.data_ptr(), a.rays, d_t.data_ptr(), d_id.data_ptr(),
                                     d_hit.data_ptr())
            ctx.synchronize()
            print("closest %d rays vs %d tris rep %d: %.2f ms (host clock)"
                  % (a.rays, a.n, i, (time.perf_counter() - t0) * 1e3))


def run_batch(a):
    specs = scenes.batch_specs(count=a.scenes, master_seed=7, tri_min=1000, tri_max=a.tri_max)
    with pt.Batch() as b:
        for sp in specs:
            sh, lc, cam = scenes.scene_from_spec(sp)
            b.add(sh, lc, cam, sp["res"], sp["res"], sp["spp"], pt.make_seeds(sp["seed"], 2 * sp["res"] ** 2),
                  max_depth=6)
        b.build(abi.FLAG_TREELET | abi.treelet_sweeps(2))
        print("batch build %.2f ms (device)" % b.info()["build_ms"])
        for i in range(a.frames):
            t0 = time.perf_counter()
            b.reset()
            b.render()
            print("batch %d scenes frame %d: %.2f ms (host clock)" % (len(specs), i, (time.perf_counter() - t0) * 1e3))


def run_kd(a):
    shapes, lc, _ = scenes.icosphere_scene(level=6)
    with pt.Context(8, 8, accel=abi.ACCEL_KDTREE) as ctx:
        ctx.set_shapes(shapes, lc)
        for i in range(a.builds):
            ctx.build(abi.ACCEL_KDTREE)
            print("kd build %d: %.3f ms" % (i, ctx.last_build_ms()))


def run_ingest(a):
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        path = scenes.write_model_scene(d, a.n, seed=11)
        for i in range(a.reps):
            with pt.Context(8, 8) as ctx:
                t0 = time.perf_counter()
                ctx.stream_scene(path)
                print("stream_scene %d shapes rep %d: %.2f ms (host clock)"
                      % (ctx.n, i, (time.perf_counter() - t0) * 1e3))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["render", "lbvh", "closest", "batch", "kd", "ingest", "scene_build"])
    ap.add_argument("--width", type=int, default=512)
    ap.add_argument("--height", type=int, default=512)
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--max-depth", type=int, default=8)
    ap.add_argument("--frames", type=int, default=2)
    ap.add_argument("--flags", type=int, default=0, help="ptgpu_config.flags of the render context")
    ap.add_argument("--sweeps", type=int, default=2, help="treelet rounds of the scene build")
    ap.add_argument("--accel", default="bvh", choices=["bvh", "kd"], help="render: the tree traversed")
    ap.add_argument("--n", type=int, default=1 << 22)
    ap.add_argument("--builds", type=int, default=2)
    ap.add_argument("--rays", type=int, default=1 << 24)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--scenes", type=int, default=16)
    ap.add_argument("--tri-max", type=int, default=200_000)
    a = ap.parse_args()
    if a.case == "ingest" and a.n == 1 << 22:
        a.n = 1_000_000
    {"render": run_render, "lbvh": run_lbvh, "closest": run_closest, "batch": run_batch, "kd": run_kd,
     "scene_build": run_scene_build,
     "ingest": run_ingest}[a.case](a)


if __name__ == "__main__":
    main()
