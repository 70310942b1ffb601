// trace.cu -- closest-hit queries and the per-pixel radiance path tracer.
//
// The tracer (RadianceGPU, rendering_kernel.cl:1072-1150, with
// RadiancePathTracing / RadianceOnePathTracing / SampleLights) runs as a
// per-lane state machine around one resumable traversal.  Each lane has at
// most one ray query in flight -- an extension ray or one light's shadow ray
// -- held in a Trav record with its own stack.  A warp advances its queries
// one traversal step (a leaf's primitives, then a node's children) at a
// time, and leaves the stepping loop only when a set share of its live
// lanes (PTGPU_RENDER_REFILL / 32) has an answered query or none: those
// lanes then consume their answers and start their next queries together,
// while the other lanes keep their place in their traversals.  Lanes thus
// stay busy in the traversal instead of idling until the warp's longest
// query ends, and the shading code runs for many lanes at once.  A lane that
// has finished all passes of its pixel takes the next pixel from a global
// counter: the lanes that need work vote (ballot), one atomicAdd reserves a
// contiguous run, and each lane's slot is its prefix popcount in the vote.
//
// A pixel's passes are sequential by construction -- each continues the
// pixel's seed stream where the previous one stopped -- so one lane runs all
// of a pixel's passes and keeps its seeds and running mean in registers.
// Deferring a query changes no random draw and no result: SampleLights
// consumes its two randoms before the visibility test, the light
// contributions are summed in light order as in the reference, and every
// query visits its nodes in the same order whether it runs in one go or in
// steps.
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"
#include "lbvh.h"

namespace ptgpu {

template <bool WIDE>
__global__ void __launch_bounds__(128) k_trace_closest(TraceView tv,
                                                        const ptgpu_ray *__restrict__ rays, int n,
                                                        float *__restrict__ tout,
                                                        uint32_t *__restrict__ idout,
                                                        int32_t *__restrict__ hitout) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *rp = reinterpret_cast<const float *>(rays + i);
    f3 o = mk3(rp[0], rp[1], rp[2]);
    f3 d = mk3(rp[3], rp[4], rp[5]);
    float t;
    int prim;
    int h = trace_query<WIDE, false>(tv, o, d, false, 0.f, t, prim, nullptr);
    tout[i] = t;
    idout[i] = (h && prim >= 0) ? (uint32_t)__ldg(&tv.prim_id[prim]) : 0u;
    hitout[i] = h;
}

__device__ __forceinline__ uint32_t to_int(float x) {
    return (uint32_t)(int)(powf(cl_clamp(x, 0.f, 1.f), 1.f / 2.2f) * 255.f + .5f);
}

enum : int { ST_NEED = 0, ST_GEN = 1, ST_EXT = 2, ST_NEE = 3, ST_DONE = 4 };

#ifndef PTGPU_RENDER_SMEM_STATE
#define PTGPU_RENDER_SMEM_STATE 1   // 72 -> 64 registers, 8 CTAs per SM: 28.73 -> 28.58 ms per frame
#endif
#ifndef PTGPU_RENDER_MINBLOCKS
// 8 CTAs of 128 lanes per SM, at most 64 registers (no spills); against 7:
// 28.80 vs 28.88 ms per benchmark frame, 260.4 vs 275.5 ms per 16-scene
// batched frame; 9 (56 registers, 60 bytes spilled): 29.60 vs 28.75 ms
#define PTGPU_RENDER_MINBLOCKS 8
#endif
#ifndef PTGPU_RENDER_BATCH_MINBLOCKS
// the batched tracer at 9 CTAs per SM (56 registers, 124 bytes spilled): a
// 16-scene batched frame 252.6 against 260.4 ms at 8
#define PTGPU_RENDER_BATCH_MINBLOCKS 9
#endif
// A warp leaves its traversal steps to shade when at least this many 32nds
// of its live lanes wait without a query in flight (32: when every query of
// the warp is answered).
#ifndef PTGPU_RENDER_REFILL
#define PTGPU_RENDER_REFILL 22
#endif
// traversal steps between two looks at the warp's waiting lanes
#ifndef PTGPU_RENDER_STEPS
#define PTGPU_RENDER_STEPS 1
#endif
// The tracer proper.  BATCH: the lanes' pixels come from many scenes (scene
// records in a.scenes, hand-out offsets in a.pix_start); otherwise from the
// one scene of the single-scene fields.  STACK: traversal stack entries.
constexpr int kMaxBatchScenes = 256;

template <bool WIDE, bool COUNT, bool BATCH, int STACK>
__global__ void __launch_bounds__(128, BATCH ? PTGPU_RENDER_BATCH_MINBLOCKS : PTGPU_RENDER_MINBLOCKS) k_render(const RenderArgs a, unsigned int *pixel_counter) {
    __shared__ int64_t s_start[BATCH ? kMaxBatchScenes + 1 : 1];
    int64_t npx;
    if (BATCH) {
        for (int i = threadIdx.x; i <= a.n_scenes; i += blockDim.x) s_start[i] = a.pix_start[i];
        __syncthreads();
        npx = s_start[a.n_scenes];
    } else {
        npx = (int64_t)a.width * a.height;
    }
    const int lane = threadIdx.x & 31;
    const int refill = a.refill > 0 ? a.refill : PTGPU_RENDER_REFILL;
    int state = ST_NEED;
    int gid = 0, passes_done = 0, depth = 0, li = 0, specular = 1;
    // a pixel's work for the next frame's hand-out order: SM clock cycles from
    // taking the pixel to finishing it (PTGPU_ORDER_CLOCK=0: loop rounds, which
    // ordered the benchmark frame no better than row order; cycles: 29.5 ->
    // 28.8 ms)
#ifndef PTGPU_ORDER_CLOCK
#define PTGPU_ORDER_CLOCK 1
#endif
    uint32_t work = 0;   // loop rounds spent on the lane's pixel
    uint32_t t_pix = 0;  // SM clock when the lane took its pixel
    int sc = 0;          // BATCH: the lane's scene (hand-out order)
    uint32_t s0 = 0, s1 = 0;
#if PTGPU_RENDER_SMEM_STATE
    // the lane's colour and hit state lives in shared memory (12-byte
    // stride: lane i on bank 3i mod 32, no conflicts): it is touched when a
    // query is made or consumed, not while the traversal steps, and its 21
    // registers would otherwise be held through every step
    __shared__ f3 s_lane[7][128];
    f3 &col = s_lane[0][threadIdx.x], &rad = s_lane[1][threadIdx.x], &tp = s_lane[2][threadIdx.x];
    f3 &hp = s_lane[3][threadIdx.x], &nl = s_lane[4][threadIdx.x], &ld = s_lane[5][threadIdx.x];
    f3 &pend = s_lane[6][threadIdx.x];
    col = mk3(0.f, 0.f, 0.f); rad = col; tp = col; hp = col; nl = col; ld = col; pend = col;
#else
    f3 col = mk3(0.f, 0.f, 0.f), rad = col, tp = col, hp = col, nl = col;
    f3 ld = col, pend = col;
#endif
    Trav q;
    q.o = col; q.d = col; q.inv = col; q.tb = 0.f; q.prim = -1; q.cur = 0; q.ccnt = 0; q.sp = 0;
    q.any = 0; q.hit = 0;
    int skip = a.tv.n_shapes - 1;   // the shape shadow queries never test (BATCH: the lane's scene's)
#if PTGPU_RENDER_SHORT_STACK > 0
    // the bottom of each lane's traversal stack in shared memory, the rest in
    // local memory (ShortStack)
    __shared__ int s_stack[PTGPU_RENDER_SHORT_STACK][128];
    ShortStack<STACK, PTGPU_RENDER_SHORT_STACK, 128> stack;
    stack.sh = &s_stack[0][threadIdx.x];
#else
    LocalStack<STACK> stack;
#endif
    bool trav = false;   // a query in flight
    bool fin = false;    // an answered query not yet consumed
    Counts cnt[3] = {{0, 0}, {0, 0}, {0, 0}};

    // per-scene values: from the lane's scene record, or the single scene's
    auto S = [&]() -> const BatchScene & { return a.scenes[sc]; };
    auto width = [&]() { return BATCH ? __ldg(&S().width) : a.width; };
    auto height = [&]() { return BATCH ? __ldg(&S().height) : a.height; };
    auto pix_off = [&]() -> int64_t { return BATCH ? __ldg(&S().pix_off) : 0; };
    auto max_depth = [&]() { return BATCH ? __ldg(&S().max_depth) : a.max_depth; };
    auto n_lights = [&]() { return BATCH ? __ldg(&S().n_lights) : a.n_lights; };
    auto start_sample = [&]() { return BATCH ? __ldg(&S().start_sample) : a.start_sample; };
    auto passes = [&]() { return BATCH ? __ldg(&S().passes) : a.passes; };

    // Optional throughput Russian roulette (RenderArgs::rr_depth > 0, single
    // scene only): called when a path is about to continue past a hit, with
    // `depth` already the next segment's; from the hit at depth rr_depth on
    // it draws one random and ends the path with probability 1 - p,
    // p = min(max(throughput), 1), or divides the throughput by p.
    auto rr_stop = [&]() -> bool {
        if (BATCH || a.rr_depth <= 0 || depth - 1 < a.rr_depth) return false;
        const float u = get_random(s0, s1);
        const float pr = fminf(fmaxf(tp.x, fmaxf(tp.y, tp.z)), 1.f);
        if (!(u < pr)) return true;
        tp = smul3(1.f / pr, tp);
        return false;
    };

    // starts a query; an immediately answered one is consumed like any other
    auto start = [&](f3 o, f3 d, bool any, float maxt) {
        Counts *c = cnt + (any ? 1 : 0);
        TraceRoot root;
        if (BATCH) {
            root.first = __ldg(&S().root);
            root.count = 0;
            root.n_shapes = __ldg(&S().n_shapes);
            root.skip = __ldg(&S().skip);
            root.box = S().root_box;
            skip = root.skip;
        } else {
            root = view_root(a.tv);
        }
        if (trav_begin<COUNT>(a.tv, root, q, o, d, any, maxt, c)) fin = true;
        else trav = true;
    };

    for (;;) {
        // ---- refill lanes that finished their pixel
        const bool need = state == ST_NEED;
        const unsigned nm = __ballot_sync(0xffffffffu, need);
        if (nm) {
            const int leader = __ffs(nm) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(pixel_counter, (unsigned)__popc(nm));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need) {
                const int64_t g = (int64_t)base + __popc(nm & ((1u << lane) - 1u));
                if (g >= npx) {
                    state = ST_DONE;
                } else {
                    if (BATCH) {   // the scene whose hand-out range holds g
                        int lo = 0, hi = a.n_scenes - 1;
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (s_start[mid] <= g) lo = mid; else hi = mid - 1;
                        }
                        sc = lo;
                        gid = (int)(g - s_start[lo]);
                    } else {
                        gid = a.order ? __ldg(a.order + g) : (int)g;
                    }
                    work = 0;
                    if (PTGPU_ORDER_CLOCK) t_pix = (uint32_t)clock();
                    const uint2 sd = reinterpret_cast<const uint2 *>(a.seeds)[pix_off() + gid];
                    s0 = sd.x; s1 = sd.y;
                    if (start_sample() > 0) {
                        const int w = width(), h = height();
                        const int x = gid % w, y = gid / w;
                        const ptgpu_vec c = a.colors[pix_off() + (int64_t)(h - y - 1) * w + x];
                        col = mk3(c.x, c.y, c.z);
                    }
                    passes_done = 0;
                    state = ST_GEN;
                }
            }
        }
        if (__all_sync(0xffffffffu, state == ST_DONE)) break;
        ++work;

        // ---- lanes without a query: produce the next one
        if (!trav && !fin) {
            if (state == ST_GEN) {
                // GenerateCameraRay (rendering_kernel.cl:1042-1070)
                const int w = width(), h = height();
                const float inv_w = 1.f / (float)w, inv_h = 1.f / (float)h;
                const int x = gid % w, y = gid / w;
                const ptgpu_camera &cam = BATCH ? S().cam : a.cam;
                const float r1 = get_random(s0, s1) - .5f;
                const float r2 = get_random(s0, s1) - .5f;
                const float kcx = ((float)x + r1) * inv_w - .5f;
                const float kcy = ((float)y + r2) * inv_h - .5f;
                f3 rdir = mk3(cam.x.x * kcx + cam.y.x * kcy + cam.dir.x,
                              cam.x.y * kcx + cam.y.y * kcy + cam.dir.y,
                              cam.x.z * kcx + cam.y.z * kcy + cam.dir.z);
                const f3 o = add3(smul3(0.1f, rdir), mk3(cam.orig.x, cam.orig.y, cam.orig.z));
                rad = mk3(0.f, 0.f, 0.f);
                tp = mk3(1.f, 1.f, 1.f);
                specular = 1;
                depth = 0;
                state = ST_EXT;
                if (COUNT) cnt[2].p++;
                start(o, norm3(rdir), false, 0.f);
            } else if (state == ST_NEE) {
                // SampleLights (rendering_kernel.cl:397-493): the next light
                // that needs a visibility test
                bool has_q = false;
                const int nlights = n_lights();
                const LightRec *lights = BATCH ? a.lights + __ldg(&S().light_first) : a.lights;
                while (li < nlights) {
                    const LightRec L = lights[li];
                    float u1, u2;
                    if (a.rtl) { u2 = get_random(s0, s1); u1 = get_random(s0, s1); }
                    else       { u1 = get_random(s0, s1); u2 = get_random(s0, s1); }
                    f3 lp, lnrm;
                    if (__float_as_int(L.a.w) == PTGPU_TRIANGLE) {
                        const float su1 = sqrtf(u1);
                        const float bu = 1.0f - su1, bv = u2 * su1;
                        const f3 e1 = smul3(bu, mk3(L.b.x, L.b.y, L.b.z));
                        const f3 e2 = smul3(bv, mk3(L.c.x, L.c.y, L.c.z));
                        lp = add3(add3(mk3(L.a.x, L.a.y, L.a.z), e1), e2);
                        lnrm = norm3(cross3(e1, e2));
                    } else {
                        const float zz = 1.f - 2.f * u1;
                        const float rr = sqrtf(fmaxf(0.f, 1.f - zz * zz));
                        const float phi = 2.f * kPi * u2;
                        float sphi, cphi;
                        pt_sincos(phi, sphi, cphi);
                        const f3 unit = mk3(rr * cphi, rr * sphi, zz);
                        lp = add3(smul3(L.b.x, unit), mk3(L.a.x, L.a.y, L.a.z));
                        lnrm = unit;
                    }
                    f3 sd = sub3(lp, hp);
                    const float len = sqrtf(dot3(sd, sd));
                    sd = smul3(1.f / len, sd);
                    float wo = dot3(sd, lnrm);
                    if (wo > 0.f) { ++li; continue; }
                    wo = -wo;
                    wo = cl_clamp(wo, 0.f, 1.f);
                    const float wi = dot3(sd, nl);
                    if (wi > 0.f) {
                        const float s = L.b.w * wi * wo / (len * len);
                        pend = smul3(s, mk3(L.e.x, L.e.y, L.e.z));
                        has_q = true;
                        if (COUNT) cnt[2].v++;
                        start(hp, sd, true, len - kEps);
                        break;
                    }
                    ++li;
                }
                if (!has_q) {
                    // all lights done: Ld * throughput, then the diffuse bounce
                    ld = mul3(ld, tp);
                    rad = add3(rad, ld);
                    const float r1 = 2.f * kPi * get_random(s0, s1);
                    const float r2 = get_random(s0, s1);
                    const float r2s = sqrtf(r2);
                    f3 w = nl;
                    const f3 av = (fabsf(w.x) > .1f) ? mk3(0.f, 1.f, 0.f) : mk3(1.f, 0.f, 0.f);
                    f3 u = norm3(cross3(av, w));
                    f3 v = cross3(w, u);
                    float sr1, cr1;
                    pt_sincos(r1, sr1, cr1);
                    u = smul3(cr1 * r2s, u);
                    v = smul3(sr1 * r2s, v);
                    f3 nd = add3(u, v);
                    w = smul3(sqrtf(1.f - r2), w);
                    nd = add3(nd, w);
                    if (++depth > max_depth() || rr_stop()) {
                        state = -1;   // pass finished
                    } else {
                        state = ST_EXT;
                        if (COUNT) cnt[2].p++;
                        start(hp, nd, false, 0.f);
                    }
                }
            }
        }

        // ---- traversal steps, until enough lanes wait to be served
        for (;;) {
            const unsigned busy = __ballot_sync(0xffffffffu, trav);
            if (!busy) break;
            const unsigned live = __ballot_sync(0xffffffffu, state != ST_DONE);
            if (__popc(live & ~busy) * 32 >= refill * __popc(live)) break;
            if (trav && trav_step<WIDE, COUNT, STACK>(a.tv, q, stack, cnt + q.any, skip)) {
                trav = false;
                fin = true;
            }
#if PTGPU_RENDER_STEPS > 1
            if (trav && trav_step<WIDE, COUNT, STACK>(a.tv, q, stack, cnt + q.any, skip)) {
                trav = false;
                fin = true;
            }
#endif
        }

        // ---- consume answered queries
        if (fin) {
            fin = false;
            if (q.any) {
                if (!q.hit) ld = add3(ld, pend);
                ++li;
            } else if (!q.hit) {
                // RadianceOnePathTracing (rendering_kernel.cl:495-753)
                state = -1;
            } else {
                const f3 d = q.d;
                hp = add3(q.o, smul3(q.tb, d));
                const int prim = q.prim;
                const int shape0 = BATCH ? __ldg(&S().shape0) : 0;
                const int id = prim >= 0 ? __ldg(&a.tv.prim_id[prim]) : shape0;
                const Material m = a.mats[id];
                const int type = __float_as_int(m.e_type.w);
                const float4 *pp = prim >= 0 ? a.tv.prims : a.prims0;
                const int k = prim >= 0 ? prim : shape0;
                const float4 g0 = __ldg(&pp[3 * k + 0]);
                f3 normal;
                if (type == PTGPU_SPHERE) {
                    normal = sub3(hp, mk3(g0.x, g0.y, g0.z));
                } else {
                    const float4 g1 = __ldg(&pp[3 * k + 1]);
                    const float4 g2 = __ldg(&pp[3 * k + 2]);
                    normal = cross3(mk3(g1.x, g1.y, g1.z), mk3(g2.x, g2.y, g2.z));
                }
                normal = norm3(normal);
                const float dp = dot3(normal, d);
                const float inv_sign = -1.f * cl_sign(dp);
                nl = smul3(inv_sign, normal);
                f3 ecol = mk3(m.e_type.x, m.e_type.y, m.e_type.z);
                const f3 colr = mk3(m.c_refl.x, m.c_refl.y, m.c_refl.z);
                const int refl = __float_as_int(m.c_refl.w);
                if (!iszero3(ecol)) {
                    if (specular) {
                        ecol = smul3(fabsf(dp), ecol);
                        ecol = mul3(tp, ecol);
                        rad = add3(rad, ecol);
                    }
                    state = -1;
                } else if (refl == PTGPU_DIFF) {
                    specular = 0;
                    tp = mul3(tp, colr);
                    ld = mk3(0.f, 0.f, 0.f);
                    li = 0;
                    state = ST_NEE;
                } else {
                    specular = 1;
                    f3 nd;
                    if (refl == PTGPU_SPEC) {
                        nd = sub3(d, smul3(2.f * dot3(normal, d), normal));
                        tp = mul3(tp, colr);
                    } else {
                        const f3 refl_d = sub3(d, smul3(2.f * dot3(normal, d), normal));
                        const bool into = dot3(normal, nl) > 0;
                        const float nc = 1.f, nt = 1.5f;
                        const float nnt = into ? nc / nt : nt / nc;
                        const float ddn = dot3(d, nl);
                        const float cos2t = 1.f - nnt * nnt * (1.f - ddn * ddn);
                        if (cos2t < 0.f) {
                            tp = mul3(tp, colr);
                            nd = refl_d;
                        } else {
                            const float kk = (float)(into ? 1 : -1) * (ddn * nnt + sqrtf(cos2t));
                            const f3 nkk = smul3(kk, normal);
                            const f3 tdir = norm3(sub3(smul3(nnt, d), nkk));
                            const float aa = nt - nc, bb = nt + nc;
                            const float R0 = aa * aa / (bb * bb);
                            const float c = 1.f - (into ? -ddn : dot3(tdir, normal));
                            const float Re = R0 + (1.f - R0) * c * c * c * c * c;
                            const float Tr = 1.f - Re;
                            const float P = .25f + .5f * Re;
                            const float RP = Re / P;
                            const float TP = Tr / (1.f - P);
                            if (get_random(s0, s1) < P) {
                                tp = smul3(RP, tp);
                                tp = mul3(tp, colr);
                                nd = refl_d;
                            } else {
                                tp = smul3(TP, tp);
                                tp = mul3(tp, colr);
                                nd = tdir;
                            }
                        }
                    }
                    if (++depth > max_depth() || rr_stop()) {
                        state = -1;
                    } else {
                        if (COUNT) cnt[2].p++;
                        start(hp, nd, false, 0.f);
                    }
                }
            }
        }

        // ---- a finished pass: running mean, next pass or next pixel
        if (state == -1) {
            const int cs = start_sample() + passes_done;
            if (cs == 0) {
                col = rad;
            } else {
                const float k1 = (float)cs;
                const float k2 = 1.f / ((float)cs + 1.f);
                col.x = (col.x * k1 + rad.x) * k2;
                col.y = (col.y * k1 + rad.y) * k2;
                col.z = (col.z * k1 + rad.z) * k2;
            }
            if (++passes_done < passes()) {
                state = ST_GEN;
            } else {
                const int w = width(), h = height();
                const int x = gid % w, y = gid / w;
                const int64_t po = pix_off();
                ptgpu_vec out;
                out.x = col.x; out.y = col.y; out.z = col.z;
                a.colors[po + (int64_t)(h - y - 1) * w + x] = out;
                a.pixels[po + gid] = to_int(col.x) | (to_int(col.y) << 8) | (to_int(col.z) << 16) |
                                     0xff000000u;
                reinterpret_cast<uint2 *>(a.seeds)[po + gid] = make_uint2(s0, s1);
                if (!BATCH && a.cost) a.cost[gid] = PTGPU_ORDER_CLOCK ? (uint32_t)clock() - t_pix : work;
                state = ST_NEED;
            }
        }
    }
    if (COUNT) {
        atomicAdd(a.stats + 0, (unsigned long long)cnt[0].v);
        atomicAdd(a.stats + 1, (unsigned long long)cnt[0].p);
        atomicAdd(a.stats + 2, (unsigned long long)cnt[1].v);
        atomicAdd(a.stats + 3, (unsigned long long)cnt[1].p);
        atomicAdd(a.stats + 4, (unsigned long long)cnt[2].p);
        atomicAdd(a.stats + 5, (unsigned long long)cnt[2].v);
    }
}

static int resident_grid(const void *kernel, int block, int max_ctas) {
    int per_sm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
    int resident = per_sm * sms;
    if (max_ctas > 0 && resident > max_ctas) resident = max_ctas;
    return resident;
}

// ---- hand-out order of the next frame -----------------------------------
// class of a pixel's work: 0 for the most, kOrderClasses - 1 for the least
// (kOrderSub classes per power of two)
#ifndef PTGPU_ORDER_SUBBITS
#define PTGPU_ORDER_SUBBITS 3
#endif
constexpr int kOrderSub = 1 << PTGPU_ORDER_SUBBITS;
constexpr int kOrderClasses = 32 * kOrderSub;
static_assert(kOrderClasses <= kOrderScratchWords, "order scratch");
__device__ __forceinline__ int work_class(uint32_t w) {
    const uint32_t v = w + 1u;
    const int lz = 31 - __clz((int)v);
    const int sub = lz >= PTGPU_ORDER_SUBBITS ? (int)((v >> (lz - PTGPU_ORDER_SUBBITS)) & (kOrderSub - 1))
                                              : (int)((v << (PTGPU_ORDER_SUBBITS - lz)) & (kOrderSub - 1));
    return kOrderClasses - 1 - (kOrderSub * lz + sub);
}

__global__ void k_order_hist(const uint32_t *__restrict__ cost, int npx, uint32_t *__restrict__ hist) {
    __shared__ uint32_t h[kOrderClasses];
    for (int i = threadIdx.x; i < kOrderClasses; i += blockDim.x) h[i] = 0u;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npx; i += gridDim.x * blockDim.x)
        atomicAdd(&h[work_class(__ldg(cost + i))], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < kOrderClasses; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// hist[0..C-1] -> exclusive offsets in hist[C..2C-1] (one block of C threads)
__global__ void k_order_scan(uint32_t *hist) {
    __shared__ uint32_t t[kOrderClasses];
    const int c = threadIdx.x;
    t[c] = hist[c];
    __syncthreads();
    for (int o = 1; o < kOrderClasses; o <<= 1) {      // inclusive Hillis-Steele scan
        const uint32_t v = c >= o ? t[c - o] : 0u;
        __syncthreads();
        t[c] += v;
        __syncthreads();
    }
    hist[kOrderClasses + c] = t[c] - hist[c];
}

__global__ void k_order_scatter(const uint32_t *__restrict__ cost, int npx, uint32_t *__restrict__ offs,
                                int32_t *__restrict__ order) {
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x; base < npx; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        const bool ok = i < npx;
        const int c = ok ? work_class(__ldg(cost + i)) : kOrderClasses + lane;   // distinct dummies
        const unsigned peers = __match_any_sync(0xffffffffu, c);
        const int leader = __ffs(peers) - 1;
        uint32_t pos = 0;
        if (ok && lane == leader) pos = atomicAdd(&offs[c], (uint32_t)__popc(peers));
        pos = __shfl_sync(0xffffffffu, pos, leader);
        if (ok) order[pos + __popc(peers & ((1u << lane) - 1u))] = i;
    }
}

cudaError_t launch_pixel_order(const uint32_t *cost, int32_t *order, uint32_t *scratch, int npx, cudaStream_t s) {
    if (npx <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scratch, 0, kOrderClasses * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = std::min((npx + 255) / 256, sms * 4);
    k_order_hist<<<grid, 256, 0, s>>>(cost, npx, scratch);
    k_order_scan<<<1, kOrderClasses, 0, s>>>(scratch);
    k_order_scatter<<<grid, 256, 0, s>>>(cost, npx, scratch + kOrderClasses, order);
    return cudaGetLastError();
}

cudaError_t launch_render(const RenderArgs &a, int block, cudaStream_t s) {
    const int n = a.width * a.height;
    if (n <= 0 || a.passes <= 0) return cudaSuccess;
    if (block <= 0) block = 128;
    if (!a.pixel_counter) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(a.pixel_counter, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    // lanes pull pixels until none remain; the grid is capped at what is resident
    const bool wide = a.tv.nodes4 != nullptr;
    int grid = (n + block - 1) / block;
    int resident = wide ? resident_grid((const void *)k_render<true, false, false, kStackSize>, block, a.max_ctas)
                        : resident_grid((const void *)k_render<false, false, false, kStackSize>, block, a.max_ctas);
#ifdef PTGPU_RENDER_GRID
    if (resident > PTGPU_RENDER_GRID) resident = PTGPU_RENDER_GRID;
#endif
    if (resident > 0 && grid > resident) grid = resident;
    if (a.stats) {
        if (wide) k_render<true, true, false, kStackSize><<<grid, block, 0, s>>>(a, a.pixel_counter);
        else k_render<false, true, false, kStackSize><<<grid, block, 0, s>>>(a, a.pixel_counter);
    } else {
        if (wide) k_render<true, false, false, kStackSize><<<grid, block, 0, s>>>(a, a.pixel_counter);
        else k_render<false, false, false, kStackSize><<<grid, block, 0, s>>>(a, a.pixel_counter);
    }
    return cudaGetLastError();
}

// A batched render over a.n_scenes scene records (binary nodes only).  The
// pixel counter is cleared on the stream first, so the pair can be captured
// into a graph and replayed.
int render_stack_for_depth(int depth) {
    const int words = 2 * depth + 2;   // at most one push of <= 2 words per level
    return words <= 32 ? 32 : (words <= 64 ? 64 : 128);
}

int render_batch_grid(int block, int stack, int max_ctas) {
    const void *k = stack > 64 ? (const void *)k_render<false, false, true, 128>
                  : stack > 32 ? (const void *)k_render<false, false, true, 64>
                               : (const void *)k_render<false, false, true, 32>;
    return resident_grid(k, block > 0 ? block : 128, max_ctas);
}

cudaError_t launch_render_batch(const RenderArgs &a, int block, int stack, int grid, cudaStream_t s) {
    if (!a.scenes || !a.pix_start || a.n_scenes <= 0 || a.n_scenes > kMaxBatchScenes)
        return cudaErrorInvalidValue;
    if (block <= 0) block = 128;
    if (!a.pixel_counter || grid <= 0) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(a.pixel_counter, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    if (a.stats) {
        if (stack > 64) k_render<false, true, true, 128><<<grid, block, 0, s>>>(a, a.pixel_counter);
        else if (stack > 32) k_render<false, true, true, 64><<<grid, block, 0, s>>>(a, a.pixel_counter);
        else k_render<false, true, true, 32><<<grid, block, 0, s>>>(a, a.pixel_counter);
    } else {
        if (stack > 64) k_render<false, false, true, 128><<<grid, block, 0, s>>>(a, a.pixel_counter);
        else if (stack > 32) k_render<false, false, true, 64><<<grid, block, 0, s>>>(a, a.pixel_counter);
        else k_render<false, false, true, 32><<<grid, block, 0, s>>>(a, a.pixel_counter);
    }
    return cudaGetLastError();
}

// Closest hits of a ray batch with persistent lanes: each lane takes the
// next ray from a global counter (one atomicAdd per warp), and a warp steps
// its rays' traversals until `refill`/32 of its live lanes are idle, then
// writes their results and refills them together -- the render kernel's
// schedule without the shading.  Each ray visits its nodes in the same order
// as in trace_query.
// COUNT: node visits and primitive tests summed into stats[0..1].
template <bool WIDE, bool COUNT>
// Binary nodes: 12 resident CTAs of 128 lanes per SM (40 registers, 8 bytes
// spilled) instead of 10 at 47: 2^24 random rays against 4M triangles
// 24.5 -> 20.6 ms.  The 4-wide traversal keeps its own register count (at 12
// CTAs it would spill 126 bytes; not measured).
#ifndef PTGPU_CLOSEST_MINBLOCKS
#define PTGPU_CLOSEST_MINBLOCKS 12
#endif
__global__ void __launch_bounds__(128, WIDE ? 1 : PTGPU_CLOSEST_MINBLOCKS) k_trace_closest_p(TraceView tv,
                                                          const ptgpu_ray *__restrict__ rays,
                                                          int n, float *__restrict__ tout,
                                                          uint32_t *__restrict__ idout,
                                                          int32_t *__restrict__ hitout,
                                                          unsigned int *counter, int refill,
                                                          unsigned long long *stats) {
    const int lane = threadIdx.x & 31;
    Counts cnt = {0, 0};
    const TraceRoot root = view_root(tv);
    Trav q;
    q.tb = 0.f; q.prim = -1; q.cur = 0; q.ccnt = 0; q.sp = 0; q.any = 0; q.hit = 0;
#if PTGPU_SHORT_STACK > 0
    __shared__ int s_stack[PTGPU_SHORT_STACK][128];
    ShortStack<kStackSize, PTGPU_SHORT_STACK, 128> stack;
    stack.sh = &s_stack[0][threadIdx.x];
#else
    LocalStack<kStackSize> stack;
#endif
    int ray = -1;
    bool trav = false, fin = false, done = false;
    for (;;) {
        const bool need = !trav && !fin && !done;
        const unsigned nm = __ballot_sync(0xffffffffu, need);
        if (nm) {
            const int leader = __ffs(nm) - 1;
            unsigned base = 0;
            if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(nm));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need) {
                const int64_t r = (int64_t)base + __popc(nm & ((1u << lane) - 1u));
                if (r >= n) {
                    done = true;
                } else {
                    ray = (int)r;
                    const float *rp = reinterpret_cast<const float *>(rays + ray);
                    const f3 o = mk3(rp[0], rp[1], rp[2]);
                    const f3 d = mk3(rp[3], rp[4], rp[5]);
                    if (trav_begin<COUNT>(tv, root, q, o, d, false, 0.f, COUNT ? &cnt : nullptr)) fin = true;
                    else trav = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        for (;;) {
            const unsigned busy = __ballot_sync(0xffffffffu, trav);
            if (!busy) break;
            const unsigned live = __ballot_sync(0xffffffffu, !done);
            if (__popc(live & ~busy) * 32 >= refill * __popc(live)) break;
            if (trav && trav_step<WIDE, COUNT>(tv, q, stack, COUNT ? &cnt : nullptr, -1)) {   // closest only
                trav = false;
                fin = true;
            }
        }
        if (fin) {
            fin = false;
            tout[ray] = q.tb;
            idout[ray] = (q.hit && q.prim >= 0) ? (uint32_t)__ldg(&tv.prim_id[q.prim]) : 0u;
            hitout[ray] = q.hit;
        }
    }
    if (COUNT) {
        atomicAdd(stats + 0, (unsigned long long)cnt.v);
        atomicAdd(stats + 1, (unsigned long long)cnt.p);
    }
}

cudaError_t launch_trace_closest(const TraceView &tv, const ptgpu_ray *rays, int n, float *t,
                                 uint32_t *id, int32_t *hit, cudaStream_t s, unsigned int *counter,
                                 unsigned long long *stats) {
    if (n <= 0) return cudaSuccess;
    if (!counter) {   // one thread per ray
        if (tv.nodes4) k_trace_closest<true><<<(n + 127) / 128, 128, 0, s>>>(tv, rays, n, t, id, hit);
        else k_trace_closest<false><<<(n + 127) / 128, 128, 0, s>>>(tv, rays, n, t, id, hit);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    const void *k = tv.nodes4 ? (const void *)k_trace_closest_p<true, false>
                              : (const void *)k_trace_closest_p<false, false>;
    int grid = resident_grid(k, 128, 0);
    const int need = (n + 127) / 128;
    if (grid <= 0 || grid > need) grid = need;
    // the closest-hit lanes refill much earlier than the render's, whose
    // refill also shades: a warp takes new rays once 8 of 32 live lanes are
    // done (2^24 rays against 4M triangles: 16.76 ms at 8, 16.82 at 10, 16.95
    // at 6, 16.99 at 12, 18.71 at 20, 21.11 at 24)
#ifndef PTGPU_CLOSEST_REFILL
#define PTGPU_CLOSEST_REFILL 8
#endif
    const int r = PTGPU_CLOSEST_REFILL;
    if (stats) {
        if (tv.nodes4) k_trace_closest_p<true, true><<<grid, 128, 0, s>>>(tv, rays, n, t, id, hit, counter, r, stats);
        else k_trace_closest_p<false, true><<<grid, 128, 0, s>>>(tv, rays, n, t, id, hit, counter, r, stats);
    } else {
        if (tv.nodes4) k_trace_closest_p<true, false><<<grid, 128, 0, s>>>(tv, rays, n, t, id, hit, counter, r, nullptr);
        else k_trace_closest_p<false, false><<<grid, 128, 0, s>>>(tv, rays, n, t, id, hit, counter, r, nullptr);
    }
    return cudaGetLastError();
}

}  // namespace ptgpu
