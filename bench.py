"""Benchmark: the plain path tracer on the displaced-icosphere scene.

One step = one 512x512 frame of 16 passes (samples per pixel) at max depth 8
through the BVH, scene and tree resident in HBM, L2 flushed between steps.
value = Msamples/s over all ranks (each rank renders its own replica: the
path shards by scene/pixels with no data exchange, so N>1 is weak scaling).

Extra keys on the JSON line:
  e2e          the same metric through the C ABI with host buffers: per step
               set_shapes (H2D), BVH build, set_seeds (H2D), draw_frame
               (16 passes, D2H pixels), wall clock
  roofline     the render kernel against HBM, bytes per query after the
               closest-hit model (24 B ray + 8 B hit + 60 B per node visit +
               36 B per primitive test), counts measured by the GPU
  treelet      SAH cost, frame time and build time for 0, 1 and 2 rounds
  ingest       streamed scene ingestion of two OBJ models (1M triangles)
  batched      64 mixed scenes (1k-2M triangles, 128^2-1024^2, 1-64 passes):
               one batch (segmented build, one graph-replayed launch) against
               the same scenes rendered one by one through contexts, with the
               per-scene table and the ceiling any schedule could reach
  served       Poisson request streams over those scenes (10, 30, 100, 300 and
               1000 req/s, 70% of requests on an already requested scene):
               the server (continuous batching, 120 GB budget, LRU scene
               cache) against the plain path (first come first served, a
               context per request); throughput and p50/p99 latency
  cpu_baseline the oracle port of the reference's CPU path (C, OpenMP, all
               host threads) on a bounded sample of the same frame
  legs         lbvh (4,194,304 random triangles: Mtris/s and its HBM roofline
               at 252 algorithmic bytes per triangle), lbvh_1m, closest_hit
               (2^24 random rays against the 4M-triangle BVH), config1 (the
               9-sphere Cornell box, 256x256, 16 spp, depth 6, no
               acceleration; also with rr_depth 3), config2_kd (the
               benchmark frame through the KD tree)
  summary      the headline figure of every leg, last on the line
--impl reference times that CPU path alone (rank 0) on the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W = H = 512
SPP = 16
MAX_DEPTH = 8
LBVH_N = 1 << 22
RAYS_N = 1 << 24
INGEST_N = 1_000_000
L2_FLUSH_BYTES = 256 << 20
WORKLOAD = "icosphere_81934tri_512x512_16spp_depth8_bvh"
TREELET_ROUNDS = 2
# PTGPU_FLAG_TREELET | PTGPU_TREELET_SWEEPS(2): two rounds of the 7-leaf
# treelet stage in the scene's build
BUILD_FLAGS = 0x4 | (TREELET_ROUNDS << 8)


def ncu_traffic(profile, key):
    """DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one ncu
    capture of the same workload, from the `key: value` line of its summary
    under profiles/; None when the summary is absent."""
    try:
        with open(os.path.join(ROOT, "profiles", profile)) as f:
            for line in f:
                if line.startswith(key + ":"):
                    return int(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def issue_roofline(profile):
    """What bounds a latency- and SIMT-bound kernel: issue-active (share of
    cycles an SM sub-partition issues) times active lanes per issued warp
    instruction / 32, from the ncu summary under profiles/ (lines
    `smsp__issue_active ... %` and `smsp__thread_inst_executed_per_inst_executed
    ... of 32 lanes`); None when absent."""
    act = lanes = None
    try:
        with open(os.path.join(ROOT, "profiles", profile)) as f:
            for line in f:
                if line.startswith("smsp__issue_active"):
                    act = float(line.split()[-2]) / 100.0
                elif line.startswith("smsp__thread_inst_executed_per_inst_executed"):
                    lanes = float(line.split()[1])
    except (OSError, ValueError, IndexError):
        return None
    if act is None or lanes is None:
        return None
    return {"issue_active": act, "lanes_per_instruction": lanes, "frac": act * lanes / 32.0,
            "unit": "of lane-issue peak", "source": "profiles/" + profile}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for k, nm in enumerate(names):
                if s[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    return rank, world, local, pg


def reduce_max(value, pg, device):
    """max over ranks (a float); identity without a process group."""
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


def pinned_copy(torch, arr):
    """arr copied into page-locked host memory (same dtype and shape); the
    second value owns the memory."""
    buf = torch.empty(arr.nbytes, dtype=torch.uint8).pin_memory()
    out = buf.numpy().view(arr.dtype).reshape(arr.shape)
    out[...] = arr
    return out, buf


class CpuReference:
    """The oracle port of the reference's CPU path (the reference algorithm
    restated in C: per pixel RadiancePathTracing with the reference's
    brute-force IntersectP and its SampleLights scan of the shape list at
    every diffuse hit; OpenMP over the pixels of a row) on a bounded sample of
    the same frame: `rows` whole rows spread evenly over the frame, one pass,
    sized once so that a sample runs for about target_s seconds."""

    def __init__(self, shapes, light_cnt, cam, target_s=10.0, threads=0, w=W, h=H, depth=MAX_DEPTH,
                 accel="bvh"):
        import oracle
        from ptgpu_pc_gb300 import abi
        oracle.build()
        self.oracle = oracle
        self.shapes, self.lc = shapes, light_cnt
        self.w, self.h, self.depth = w, h, depth
        c = np.array(cam, abi.CAMERA)
        c["width"], c["height"] = w, h
        self.cam = oracle.update_camera(c)
        if accel == "bvh":
            _, btn, btl, _ = oracle.build_bvh(shapes)
            self.acc = oracle.make_accel(abi.ACCEL_BVH, btn, btl, reference_leafness=True)
        else:
            self.acc = oracle.make_accel(abi.ACCEL_NONE)
        self.accel = accel
        self.seeds = oracle.make_seeds(1, 2 * w * h)
        self.threads = threads or os.cpu_count() or 1
        self.rows = 1
        dt = self._run()
        self.rows = int(max(1, min(h, target_s / max(dt, 1e-6))))

    def _row_list(self):
        step = self.h / self.rows
        return [int(step * (k + 0.5)) for k in range(self.rows)]

    def _run(self, threads=None, cols=None):
        t0 = time.perf_counter()
        for y in self._row_list():
            self.oracle.render(self.shapes, self.lc, self.cam, self.w, self.h, self.seeds, 1,
                               accel=self.acc, max_depth=self.depth, threads=threads or self.threads,
                               rows=(y, y + 1), cols=cols, reference_cost=True)
        return time.perf_counter() - t0

    def describe(self, dt, rows=None, cols=None):
        return ("%d rows x %d pixels spread over the %dx%d frame, 1 pass, depth %d, %s, "
                "brute-force shadow rays and per-hit emitter scan as in the reference; %.2f s"
                % (rows or self.rows, cols or self.w, self.w, self.h, self.depth,
                   "BVH built by the oracle" if self.accel == "bvh" else "no acceleration", dt))

    def sample(self):
        """(Msamples/s, threads, description, seconds) of one timed sample."""
        dt = self._run()
        px = self.rows * self.w
        return px / dt / 1e6, self.threads, self.describe(dt), dt

    def sample_one_thread(self, cols=128):
        """The same port on one thread, over the first `cols` pixels of the
        sample's middle row."""
        rows = self.rows
        self.rows = 1
        try:
            dt = self._run(threads=1, cols=(0, cols))
            return cols / dt / 1e6, self.describe(dt, rows=1, cols=cols)
        finally:
            self.rows = rows


def cpu_model():
    """The host CPU's name as /proc/cpuinfo gives it (model name, or the Arm
    implementer / part codes)."""
    try:
        info = open("/proc/cpuinfo").read().splitlines()
    except OSError:
        return "unknown"
    for key in ("model name", "Model"):
        for line in info:
            if line.startswith(key):
                return line.split(":", 1)[1].strip()
    impl = [l.split(":", 1)[1].strip() for l in info if l.startswith("CPU implementer")]
    part = [l.split(":", 1)[1].strip() for l in info if l.startswith("CPU part")]
    return "implementer %s part %s" % (impl[0] if impl else "?", part[0] if part else "?")


def run_reference(args, rank, world, pg):
    """The reference arm: the CPU port of the reference's path on this machine's
    host cores (all threads), on the same workload, metric and unit as the
    GPU arm; each step is one bounded sample (whole rows spread over the
    frame), and ms_per_step is that sample's measured time."""
    from ptgpu_pc_gb300 import scenes
    if rank != 0:
        return
    shapes, lc, cam = scenes.icosphere_scene(level=6)
    per_step, secs = [], []
    desc = ""
    cores = 0
    per = max(1.0, min(args.ref_seconds, 150.0 / (args.warmup + args.steps)))
    ref = CpuReference(shapes, lc, cam, target_s=per)
    for i in range(args.warmup + args.steps):
        v, cores, desc, dt = ref.sample()
        if i >= args.warmup:
            per_step.append(v)
            secs.append(dt)
    value = float(np.mean(per_step))
    line = {"metric": "Msamples/s", "value": value, "unit": "Msamples/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(secs)) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded displaced icosphere)",
            "config": {"workload": WORKLOAD, "shapes": int(len(shapes)), "width": W, "height": H,
                       "spp": SPP, "max_depth": MAX_DEPTH, "accel": "bvh",
                       "step": "one bounded sample of the frame: %d rows x %d pixels x 1 pass"
                               % (ref.rows, W)},
            "cpu_baseline": {"value": value, "unit": "Msamples/s", "cores": cores, "kind": "port",
                             "sample": desc, "cpu": cpu_model()},
            "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_lbvh(pt, abi, scenes, torch, warmup, steps, n=None):
    """LBVH builds of n seeded random triangles (config 3's soup): device time
    of each build (CUDA events in the library), mean over `steps` after
    `warmup` builds."""
    n = n or LBVH_N
    shapes = scenes.triangle_soup(n, seed=3)
    ctx = pt.Context(8, 8)
    ctx.set_shapes(shapes, 0)
    del shapes
    times = []
    for i in range(warmup + steps):
        ctx.build(abi.ACCEL_BVH)
        if i >= warmup:
            times.append(ctx.last_build_ms())
    ms = float(np.mean(times))
    return ctx, {"metric": "LBVH Mtris/s", "n_tris": n, "value": n / ms / 1e3,
                 "unit": "Mtris/s", "ms": ms, "min_ms": float(np.min(times)), "builds": steps}


def time_frames(ctx, torch, passes, frames, flush=None):
    """Device time (CUDA events on the context's stream) of `frames` renders
    of `passes` passes each, after one warm-up frame; L2 flushed before each
    frame when `flush` (a tensor larger than L2) is given."""
    stream = torch.cuda.ExternalStream(ctx.stream())
    ctx.reset()
    ctx.render_async(passes)
    ctx.synchronize()
    ms = []
    for i in range(frames):
        if flush is not None:
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
        ctx.reset()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.render_async(passes)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return float(np.mean(ms))


def bench_config1(pt, abi, scenes, torch, flush, frames=5):
    """Config 1: the 9-sphere Cornell box, 256x256, 16 passes, depth 6, no
    acceleration structure (ACCELSTR 0); also with the opt-in throughput
    Russian roulette from depth 3 (ptgpu_config.rr_depth = 3)."""
    shapes, lc, cam = scenes.cornell_spheres()
    w = h = 256
    out = {"workload": "cornell_spheres_9_256x256_16spp_depth6_none"}
    for rr in (0, 3):
        ctx = pt.Context(w, h, accel=abi.ACCEL_NONE, max_depth=6, rr_depth=rr)
        ctx.set_shapes(shapes, lc)
        ctx.build(abi.ACCEL_NONE)
        ctx.set_camera(cam)
        ctx.set_seeds(pt.make_seeds(1, 2 * w * h))
        ms = time_frames(ctx, torch, 16, frames, flush)
        ctx.close()
        key = "value" if rr == 0 else "rr3_value"
        out[key] = w * h * 16 / ms / 1e3
        out["ms" if rr == 0 else "rr3_ms"] = ms
    out["unit"] = "Msamples/s"
    return out


def bench_config2_kd(pt, abi, shapes, lc, cam, torch, flush, frames=5):
    """Config 2 through the KD tree (ACCELSTR 2): GPU KD build with the
    reference topology, then 512x512 x 16 passes at depth 8."""
    ctx = pt.Context(W, H, accel=abi.ACCEL_KDTREE, max_depth=MAX_DEPTH)
    ctx.set_shapes(shapes, lc)
    ctx.build(abi.ACCEL_KDTREE)
    build_ms = ctx.last_build_ms()
    ctx.set_camera(cam)
    ctx.set_seeds(pt.make_seeds(1, 2 * W * H))
    ms = time_frames(ctx, torch, SPP, frames, flush)
    ctx.close()
    return {"workload": WORKLOAD.replace("_bvh", "_kd"), "value": W * H * SPP / ms / 1e3,
            "unit": "Msamples/s", "ms": ms, "kd_build_ms": build_ms}


def sah_cost(btn, btl):
    """SAH cost of a BVHNodeGPU tree (Karras & Aila 2013: Ci = 1.2 per internal
    node, Ct = 1.0 per leaf, areas relative to the root's)."""
    def area(b):                 # b: min_x, max_x, min_y, max_y, min_z, max_z per row
        b = b.astype(np.float64)
        dx, dy, dz = b[:, 1] - b[:, 0], b[:, 3] - b[:, 2], b[:, 5] - b[:, 4]
        return 2.0 * (dx * dy + dy * dz + dz * dx)
    a_in, a_lf = area(btn["bound"]), area(btl["bound"])
    return float((1.2 * a_in.sum() + 1.0 * a_lf.sum()) / a_in[0])


def bench_treelet(pt, abi, shapes, lc, cam, torch, rounds=(0, 1, 2), frames=4):
    """Treelet reoptimisation report on the benchmark scene: SAH cost of the
    tree and frame time (CUDA events, after a warm-up frame) for 0, 1 and 2
    rounds, and the build time each costs."""
    out = {"rounds": [], "sah": [], "frame_ms": [], "build_ms": []}
    for r in rounds:
        flags = (abi.FLAG_TREELET | abi.treelet_sweeps(r)) if r else 0
        with pt.Context(W, H, accel=abi.ACCEL_BVH, max_depth=MAX_DEPTH) as ctx:
            ctx.set_shapes(shapes, lc)
            ctx.build(abi.ACCEL_BVH, flags)
            build_ms = ctx.last_build_ms()
            btn, btl = ctx.get_bvh()
            ctx.set_camera(cam)
            ctx.set_seeds(pt.make_seeds(1, 2 * W * H))
            stream = torch.cuda.ExternalStream(ctx.stream())
            ms = []
            for f in range(frames + 1):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ctx.reset()
                e0.record(stream)
                ctx.render_async(SPP)
                e1.record(stream)
                e1.synchronize()
                if f > 0:
                    ms.append(e0.elapsed_time(e1))
        out["rounds"].append(r)
        out["sah"].append(sah_cost(btn, btl))
        out["frame_ms"].append(float(np.mean(ms)))
        out["build_ms"].append(build_ms)
    return out


def bench_closest(ctx, torch, scenes, warmup, steps):
    rays = scenes.random_rays(RAYS_N, seed=4)
    d_rays = torch.from_numpy(rays.view(np.uint8).reshape(-1)).cuda()
    del rays
    d_t = torch.empty(RAYS_N, dtype=torch.float32, device="cuda")
    d_id = torch.empty(RAYS_N, dtype=torch.int32, device="cuda")
    d_hit = torch.empty(RAYS_N, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream())
    ms = []
    for i in range(warmup + steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.trace_closest_device(d_rays.data_ptr(), RAYS_N, d_t.data_ptr(), d_id.data_ptr(),
                                 d_hit.data_ptr())
        e1.record(stream)
        e1.synchronize()
        if i >= warmup:
            ms.append(e0.elapsed_time(e1))
    hits = int(d_hit.sum().item())
    m = float(np.mean(ms))
    # bytes-per-ray model: 24 B ray + 8 B result + 60 B per node visit + 36 B
    # per primitive test, with visits and tests counted by the GPU (one
    # extra, untimed pass)
    visits, tests = ctx.trace_closest_stats_device(d_rays.data_ptr(), RAYS_N, d_t.data_ptr(), d_id.data_ptr(),
                                                   d_hit.data_ptr())
    model_bytes = 32 * RAYS_N + 60 * visits + 36 * tests
    return {"metric": "closest-hit Mrays/s", "rays": RAYS_N, "n_tris": LBVH_N,
            "value": RAYS_N / m / 1e3, "unit": "Mrays/s", "ms": m, "hit_fraction": hits / RAYS_N,
            "node_visits_per_ray": visits / RAYS_N, "prim_tests_per_ray": tests / RAYS_N,
            "model_bytes": model_bytes}


def bench_ingest(pt, abi, scenes, n_tris=INGEST_N, reps=3):
    """Scene-file ingestion: a seeded .txt scene with two OBJ models (n_tris
    triangles, ~38 MB of text at 1M) loaded by ptgpu_read_scene (models
    expanded into shapes on the host, then copied) and by ptgpu_stream_scene
    (vertex and index arrays copied, shapes expanded on the device).  Both
    read the OBJ files on the host threads; wall time of the call, best of
    reps, in a fresh context each time."""
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        path = scenes.write_model_scene(d, n_tris, seed=11)
        size = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d))
        best = {}
        n = 0
        for mode in ("read", "stream"):
            for _ in range(reps):
                ctx = pt.Context(8, 8)
                t0 = time.perf_counter()
                if mode == "read":
                    ctx.read_scene(path)
                else:
                    ctx.stream_scene(path)
                dt = time.perf_counter() - t0
                n = ctx.n
                ctx.close()
                best[mode] = min(best.get(mode, 1e30), dt)
    return {"metric": "scene ingestion Mshapes/s", "shapes": n, "file_bytes": size,
            "value": n / best["stream"] / 1e6, "unit": "Mshapes/s", "ms": best["stream"] * 1e3,
            "read_scene_value": n / best["read"] / 1e6, "read_scene_ms": best["read"] * 1e3,
            "host_threads": os.cpu_count()}


def served_requests(specs, n_req, rate, seed=5, hit=0.7):
    """A seeded request stream over the 64 config scenes: Poisson arrivals at
    `rate` per second; each request reuses an already requested scene with
    probability `hit` (else the next new one) and draws its resolution and
    passes from the config distribution."""
    from ptgpu_pc_gb300 import scenes
    rng = np.random.default_rng(seed)
    t, seen, nxt, out = 0.0, [], 0, []
    for i in range(n_req):
        t += rng.exponential(1.0 / rate)
        if seen and (rng.random() < hit or nxt >= len(specs)):
            sc = int(seen[rng.integers(len(seen))])
        else:
            sc = nxt
            nxt += 1
            seen.append(sc)
        res = int(rng.choice(scenes.RESOLUTIONS))
        spp = int(rng.choice(scenes.SPPS))
        out.append(dict(t=t, scene=sc, res=res, spp=spp, seed=7000 + i))
    return out


def bench_served(pt, abi, data, specs, rates=(10, 30, 100, 300, 1000), n_req=64, server_flags=0):
    """Requests arriving at each rate, served with continuous batching (one
    server, 120 GB budget, scenes resident under LRU) and, for comparison,
    by the plain path: one request after another, each building its scene in
    a fresh context.  Both produce the same pixels for a request (same seed
    streams), so the image error is equal by construction."""
    out = []
    for rate in rates:
        reqs = served_requests(specs, n_req, rate)
        samples = float(sum(r["res"] * r["res"] * r["spp"] for r in reqs))
        # served
        srv = pt.Server(budget_bytes=120 << 30, flags=server_flags)
        ids = {}
        for r in reqs:
            if r["scene"] not in ids:
                sh, lc, _ = data[r["scene"]]
                ids[r["scene"]] = srv.add_scene(sh, lc, BUILD_FLAGS)
        tickets = []
        t0 = time.perf_counter()
        for r in reqs:
            while time.perf_counter() - t0 < r["t"]:
                time.sleep(min(0.002, max(0.0, r["t"] - (time.perf_counter() - t0))))
            cam = data[r["scene"]][2]
            tickets.append(srv.submit(ids[r["scene"]], cam, r["res"], r["res"], r["spp"], r["seed"]))
        lat = []
        for tk in tickets:
            _, _, st = srv.wait(tk, want_pixels=False, want_colors=False)
            lat.append(st["latency_ms"])
        span = time.perf_counter() - t0
        info = srv.info()
        srv.close()
        # plain: first come, first served, one context per request
        plat = []
        t0 = time.perf_counter()
        for r in reqs:
            now = time.perf_counter() - t0
            if now < r["t"]:
                time.sleep(r["t"] - now)
            sh, lc, cam = data[r["scene"]]
            ctx = pt.Context(r["res"], r["res"], accel=abi.ACCEL_BVH)
            ctx.set_shapes(sh, lc)
            ctx.build(abi.ACCEL_BVH, BUILD_FLAGS)
            ctx.set_camera(cam)
            ctx.set_seeds(pt.make_seeds(r["seed"], 2 * r["res"] * r["res"]))
            ctx.draw_frame_view(r["spp"])
            ctx.close()
            plat.append((time.perf_counter() - t0 - r["t"]) * 1e3)
        pspan = time.perf_counter() - t0
        out.append({"rate_per_s": rate, "requests": n_req,
                    "value": samples / span / 1e6, "plain_value": samples / pspan / 1e6,
                    "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                    "plain_p50_ms": float(np.percentile(plat, 50)),
                    "plain_p99_ms": float(np.percentile(plat, 99)),
                    "builds": info["builds"], "steps": info["steps"],
                    "scene_hits": 1.0 - info["builds"] / n_req})
    return out


def bench_batched(pt, abi, scenes, torch, frames=2):
    """The mixed-scene workload: 64 displaced-icosphere scenes drawn from
    master seed 7 (1k-2M triangles log-uniform, 128^2..1024^2, 1..64 passes),
    max depth 6.  Batched: one Batch (segmented build, tuned, graph-replayed
    render).  Plain: the same scenes one after another through single-scene
    contexts.  Both render the same samples from the same seeds."""
    specs = scenes.batch_specs()
    data = [scenes.scene_from_spec(sp) for sp in specs]
    seeds = [pt.make_seeds(1000 + i, 2 * sp["res"] * sp["res"]) for i, sp in enumerate(specs)]
    samples = float(sum(sp["res"] * sp["res"] * sp["spp"] for sp in specs))
    shapes_total = int(sum(len(d[0]) for d in data))
    # batched
    t0 = time.perf_counter()
    b = pt.Batch()
    for (sh, lc, cam), sp, sd in zip(data, specs, seeds):
        b.add(sh, lc, cam, sp["res"], sp["res"], sp["spp"], sd)
    b.build(BUILD_FLAGS)
    build_wall = time.perf_counter() - t0
    build_ms = b.info()["build_ms"]
    b.tune()
    b.render()                                  # graph capture + warm-up
    ms = []
    for _ in range(frames):
        b.reset()
        t1 = time.perf_counter()
        b.render()
        ms.append((b.info()["render_ms"], time.perf_counter() - t1))
    info = b.info()
    b.close()
    dev_ms = float(np.mean([m[0] for m in ms]))
    frame_wall = float(np.mean([m[1] for m in ms]))
    # plain: one context per scene, in turn; per scene also its rate when
    # its frame fills the GPU (1024x1024 -- 7x the lanes the GPU holds --
    # with the scene's own passes per pixel), the best any schedule can do
    # for that scene's samples
    plain_dev_ms, plain_wall = 0.0, 0.0
    table = []
    for (sh, lc, cam), sp, sd in zip(data, specs, seeds):
        t1 = time.perf_counter()
        ctx = pt.Context(sp["res"], sp["res"], accel=abi.ACCEL_BVH)
        ctx.set_shapes(sh, lc)
        ctx.build(abi.ACCEL_BVH, BUILD_FLAGS)
        ctx.set_camera(cam)
        ctx.set_seeds(sd)
        stream = torch.cuda.ExternalStream(ctx.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.render_async(sp["spp"])
        e1.record(stream)
        e1.synchronize()
        ctx.get_pixels()
        scene_ms = e0.elapsed_time(e1)
        plain_dev_ms += scene_ms
        plain_wall += time.perf_counter() - t1
        ctx.close()
        s_i = sp["res"] * sp["res"] * sp["spp"]
        if sp["res"] >= 1024:
            full_msps = s_i / scene_ms / 1e3
        else:
            full = pt.Context(1024, 1024, accel=abi.ACCEL_BVH)
            full.set_shapes(sh, lc)
            full.build(abi.ACCEL_BVH, BUILD_FLAGS)
            full.set_camera(cam)
            full.set_seeds(pt.make_seeds(5000, 2 * 1024 * 1024))
            full_ms = time_frames(full, torch, sp["spp"], 1)
            full.close()
            full_msps = 1024 * 1024 * sp["spp"] / full_ms / 1e3
        table.append({"shapes": int(len(sh)), "res": sp["res"], "spp": sp["spp"], "samples": s_i,
                      "plain_ms": scene_ms, "plain_msps": s_i / scene_ms / 1e3, "full_msps": full_msps})
    return data, specs, {"metric": "Msamples/s", "unit": "Msamples/s",
            "workload": "64 scenes, master seed 7: %d shapes, %.1f M samples per frame, depth 6"
                        % (shapes_total, samples / 1e6),
            "value": samples / dev_ms / 1e3, "plain_value": samples / plain_dev_ms / 1e3,
            "speedup_vs_plain": plain_dev_ms / dev_ms,
            "e2e": {"value": samples / (build_wall + frame_wall) / 1e6,
                    "plain_value": samples / plain_wall / 1e6,
                    "per_step": "batched: add + segmented build + render; plain: per scene context, "
                                "upload, build, render, pixels"},
            "ceiling": {"speedup": plain_dev_ms / sum(r["samples"] / r["full_msps"] / 1e3 for r in table),
                        "how": "sum of plain per-scene render ms / sum of (scene samples / that scene's "
                               "rate on a 1024x1024 frame of its own passes, which fills the GPU)",
                        "small_scene_share": float(sum(r["samples"] for r in table if r["samples"] < 1 << 20))
                                             / samples},
            "per_scene": table,
            "render_ms": dev_ms, "plain_render_ms": plain_dev_ms, "build_ms": build_ms,
            "build_wall_s": build_wall, "frames": frames,
            "tuned": {"block": info["block"], "refill": info["refill"], "stack": info["stack"],
                      "tree_depth": info["tree_depth"]}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--no-extras", action="store_true", help="skip lbvh/closest-hit/cpu legs")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-scene batched leg")
    ap.add_argument("--served-requests", type=int, default=64,
                    help="requests per arrival rate in the served leg")
    ap.add_argument("--served-only", action="store_true",
                    help="run only the batched and served legs (the full request sweep)")
    ap.add_argument("--served-rates", default="10,30,100,300,1000",
                    help="arrival rates (requests/s) of the served leg, comma-separated")
    ap.add_argument("--served-policy", default="fill", choices=["fill", "all"],
                    help="server steps: oldest requests up to one GPU filling (fill) or every "
                         "admitted request (all)")
    args = ap.parse_args()
    rank, world, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world, pg)
        return

    import torch
    import ptgpu_pc_gb300 as pt
    from ptgpu_pc_gb300 import abi, scenes
    served_rates = tuple(float(x) for x in args.served_rates.split(","))
    server_flags = abi.SERVER_ALL_ACTIVE if args.served_policy == "all" else 0
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    if args.served_only:
        # the batching leg and the full request sweep on their own (not a
        # benchmark line: the figures behind profiles/served_sweep.md)
        data, specs, batched = bench_batched(pt, abi, scenes, torch)
        served = bench_served(pt, abi, data, specs, rates=served_rates, n_req=args.served_requests,
                              server_flags=server_flags)
        print(json.dumps({"batched": batched, "served": served}), flush=True)
        return

    shapes, lc, cam = scenes.icosphere_scene(level=6)
    ctx = pt.Context(W, H, accel=abi.ACCEL_BVH, max_depth=MAX_DEPTH, device=local)
    ctx.set_shapes(shapes, lc)
    ctx.build(abi.ACCEL_BVH, BUILD_FLAGS)     # Morton, sort, Karras, refit, treelets
    build_ms = ctx.last_build_ms()
    ctx.set_camera(cam)
    seeds = pt.make_seeds(1 + rank, 2 * W * H)
    ctx.set_seeds(seeds)
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)

    # warm-up
    for _ in range(args.warmup):
        ctx.reset()
        ctx.render_async(SPP)
    ctx.synchronize()

    # timed region: per-step events around the render launch, L2 flushed
    # between steps outside the events
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    barrier(pg)
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    launches = 0
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        ctx.reset()
        starts[i].record(stream)
        ctx.render_async(SPP)
        launches += 4        # k_render, then the next frame's hand-out order (3 kernels)
        ends[i].record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    barrier(pg)
    clk = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    dev_s = sum(step_ms) / 1e3
    dev_s_max = reduce_max(dev_s, pg, device)
    samples_all = world * W * H * SPP * args.steps
    value = samples_all / dev_s_max / 1e6

    # counters for the bytes-moved model (one extra, untimed frame)
    ctx.reset()
    st = ctx.render_stats(SPP)
    ext_v, ext_p, sh_v, sh_p, ext_q, sh_q = (int(x) for x in st)
    bytes_frame = (24 + 8) * (ext_q + sh_q) + 60 * (ext_v + sh_v) + 36 * (ext_p + sh_p)
    avg_ms = dev_s * 1e3 / args.steps
    hbm_peak, peak_kind = peaks()
    achieved = bytes_frame / (avg_ms / 1e3) / 1e9

    # e2e through the C ABI with host buffers: the step's inputs in pinned
    # host memory, copied in by the library every step
    e2e_steps = max(1, args.e2e_steps)
    ctx_e = pt.Context(W, H, accel=abi.ACCEL_BVH, max_depth=MAX_DEPTH, device=local)
    ctx_e.set_camera(cam)
    h_shapes, keep_s = pinned_copy(torch, shapes)
    h_seeds, keep_d = pinned_copy(torch, seeds)
    h2d = h_shapes.nbytes + h_seeds.nbytes
    d2h = W * H * 4
    ctx_e.set_shapes(h_shapes, lc); ctx_e.build(abi.ACCEL_BVH, BUILD_FLAGS); ctx_e.set_seeds(h_seeds)
    ctx_e.draw_frame(SPP)                     # warm-up
    barrier(pg)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx_e.set_shapes(h_shapes, lc)
        ctx_e.build(abi.ACCEL_BVH, BUILD_FLAGS)
        ctx_e.set_seeds(h_seeds)
        pix = ctx_e.draw_frame_view(SPP)
    e2e_s = reduce_max(time.perf_counter() - t0, pg, device)
    e2e_value = world * W * H * SPP * e2e_steps / e2e_s / 1e6
    ctx_e.close()

    line = {"metric": "Msamples/s", "value": value, "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": avg_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded displaced icosphere, 81,934 shapes)",
            "config": {"workload": WORKLOAD, "shapes": int(len(shapes)), "width": W, "height": H,
                       "spp": SPP, "max_depth": MAX_DEPTH, "accel": "bvh", "treelet_rounds": TREELET_ROUNDS,
                       "scene_build_ms": build_ms, "l2": "flushed between steps (256 MB write)",
                       "parallelism": "replicas x%d" % world},
            "e2e": {"value": e2e_value, "unit": "Msamples/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                    "per_step": "set_shapes + BVH build (2 treelet rounds) + set_seeds + draw_frame(16)",
                    "host_buffers": "pinned"},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak,
                         "traffic": ncu_traffic("k_render_icosphere81934_512x512_16spp.txt",
                                                "traffic_bytes_per_launch"),
                         "peak_kind": peak_kind, "kernel": "k_render",
                         "model": "bytes touched (L1/L2-served), not DRAM: per query 32 B + 60 B/node "
                                  "visit + 36 B/prim test, GPU-counted",
                         "issue": issue_roofline("k_render_icosphere81934_512x512_16spp.txt"),
                         "bytes_per_frame": bytes_frame,
                         "counts": {"ext_queries": ext_q, "shadow_queries": sh_q,
                                    "ext_node_visits": ext_v, "ext_prim_tests": ext_p,
                                    "shadow_node_visits": sh_v, "shadow_prim_tests": sh_p}},
            "clocks": clk, "wall_s": wall}
    if not args.no_extras:
        def lbvh_leg(n):
            lctx, lb = bench_lbvh(pt, abi, scenes, torch, 2, 5, n)
            lb_ach = 252 * n / (lb["ms"] / 1e3) / 1e9
            lb["roofline"] = {"bound": "hbm", "achieved": lb_ach, "peak": hbm_peak, "unit": "GB/s",
                              "frac": lb_ach / hbm_peak,
                              "traffic": ncu_traffic("lbvh_build_soup4m.txt", "traffic_bytes_per_build")
                              if n == LBVH_N else None,
                              "peak_kind": peak_kind, "model": "252 B/triangle, whole build"}
            return lctx, lb
        lctx1, lb1 = lbvh_leg(1 << 20)
        lctx1.close()
        lctx, lb = lbvh_leg(LBVH_N)
        line["treelet"] = bench_treelet(pt, abi, shapes, lc, cam, torch)
        ch = bench_closest(lctx, torch, scenes, 1, 3)
        ch_ach = ch["model_bytes"] / (ch["ms"] / 1e3) / 1e9
        ch["roofline"] = {"bound": "hbm", "achieved": ch_ach, "peak": hbm_peak, "unit": "GB/s",
                          "frac": ch_ach / hbm_peak, "peak_kind": peak_kind, "kernel": "k_trace_closest_p",
                          "model": "per ray 32 B + 60 B/node visit + 36 B/prim test, GPU-counted; "
                                   "served by L1/L2 (profiles/k_trace_closest_p_soup1m_4mrays.txt)"}
        lctx.close()
        line["ingest"] = bench_ingest(pt, abi, scenes)
        c1 = bench_config1(pt, abi, scenes, torch, flush)
        kd = bench_config2_kd(pt, abi, shapes, lc, cam, torch, flush)
        if not args.no_batched:
            data, specs, line["batched"] = bench_batched(pt, abi, scenes, torch)
            line["served"] = bench_served(pt, abi, data, specs, rates=served_rates, n_req=args.served_requests,
                                          server_flags=server_flags)
            line["served_policy"] = args.served_policy
        if rank == 0:
            cref = CpuReference(shapes, lc, cam, target_s=args.ref_seconds)
            v, cores, desc, _ = cref.sample()
            v1, desc1 = cref.sample_one_thread()
            line["cpu_baseline"] = {"value": v, "unit": "Msamples/s", "cores": cores,
                                    "kind": "port", "sample": desc, "cpu": cpu_model(),
                                    "one_thread": {"value": v1, "sample": desc1}}
        # the figures of every leg, last on the line
        summ = {"lbvh_4m": {"ms": lb["ms"], "mtris_s": lb["value"], "frac": lb["roofline"]["frac"],
                            "achieved_gbs": lb["roofline"]["achieved"],
                            "traffic": lb["roofline"]["traffic"]},
                "lbvh_1m": {"ms": lb1["ms"], "mtris_s": lb1["value"], "frac": lb1["roofline"]["frac"]},
                "closest_hit_4m_2^24": {"mrays_s": ch["value"], "ms": ch["ms"],
                                        "bytes_model_frac": ch["roofline"]["frac"]},
                "config1_spheres": {"msps": c1["value"], "rr3_msps": c1["rr3_value"]},
                "config2_kd": {"msps": kd["value"], "kd_build_ms": kd["kd_build_ms"]},
                "config2_bvh": {"msps": value, "e2e_msps": e2e_value, "scene_build_ms": build_ms}}
        if "batched" in line:
            b = line["batched"]
            summ["batched"] = {"msps": b["value"], "plain_msps": b["plain_value"],
                               "speedup": b["speedup_vs_plain"], "ceiling": b["ceiling"]["speedup"]}
            summ["served"] = [{"rate": r["rate_per_s"], "msps": r["value"], "plain_msps": r["plain_value"],
                               "p50": r["p50_ms"], "p99": r["p99_ms"], "plain_p50": r["plain_p50_ms"],
                               "plain_p99": r["plain_p99_ms"]} for r in line["served"]]
        line["legs"] = {"closest_hit": ch, "config1": c1, "config2_kd": kd, "lbvh_1m": lb1, "lbvh": lb}
        line["summary"] = summ
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
