// wavefront.cu -- the path tracer as a wavefront of small kernels.
//
// Every path slot holds one pixel (RadianceGPU's work-item).  One iteration
// advances every live path by one segment:
//   k_wf_extend   closest hit for the extension queue        (Intersect)
//   k_wf_shade    hit -> emission / miss / DIFF / SPEC / REFR (RadianceOnePathTracing);
//                 DIFF samples every light (SampleLights) into the shadow
//                 queue and draws the bounce; finished passes update the
//                 running mean and start the pixel's next pass
//   k_wf_shadow   any hit for the shadow queue                (IntersectP)
//   k_wf_resolve  Ld = sum of the visible light samples, in light order;
//                 rad += Ld * throughput; continue or finish the pass
// Queues are compacted on append: the lanes of a warp that append vote
// (ballot) or scan their counts (shuffle prefix sum), one lane reserves the
// warp's run with a single atomicAdd, each lane writes at its prefix.
// The random draws of a path happen in the reference's order (camera 2,
// per diffuse hit 2 per light then 2 for the bounce, 1 per refraction), so
// the image is the one the per-lane tracer produces.
#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"
#include "lbvh.h"

namespace ptgpu {

namespace {

constexpr int kWfThreads = 128;

__device__ __forceinline__ f3 ld3(const float4 *p, int i) {
    float4 v = p[i];
    return mk3(v.x, v.y, v.z);
}
__device__ __forceinline__ void st3(float4 *p, int i, f3 v, float w = 0.f) {
    p[i] = make_float4(v.x, v.y, v.z, w);
}

// warp-aggregated append of one element per participating lane
__device__ __forceinline__ int wf_append1(unsigned *counter, bool want) {
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (!m) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    return want ? (int)(base + __popc(m & ((1u << lane) - 1u))) : -1;
}

// warp-aggregated append of `cnt` elements per lane (shuffle prefix sum)
__device__ __forceinline__ int wf_appendn(unsigned *counter, int cnt) {
    const int lane = threadIdx.x & 31;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    unsigned base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(counter, (unsigned)total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return (int)base + incl - cnt;
}

__device__ __forceinline__ uint32_t wf_to_int(float x) {
    return (uint32_t)(int)(powf(cl_clamp(x, 0.f, 1.f), 1.f / 2.2f) * 255.f + .5f);
}

// GenerateCameraRay (rendering_kernel.cl:1042-1070) for path slot p
__device__ __forceinline__ void wf_camera(const WfArgs &a, int p, int gid, uint32_t &s0,
                                          uint32_t &s1) {
    const int x = gid % a.r.width, y = gid / a.r.width;
    const ptgpu_camera &cam = a.r.cam;
    const float inv_w = 1.f / (float)a.r.width, inv_h = 1.f / (float)a.r.height;
    const float r1 = get_random(s0, s1) - .5f;
    const float r2 = get_random(s0, s1) - .5f;
    const float kcx = ((float)x + r1) * inv_w - .5f;
    const float kcy = ((float)y + r2) * inv_h - .5f;
    f3 rdir = mk3(cam.x.x * kcx + cam.y.x * kcy + cam.dir.x,
                  cam.x.y * kcx + cam.y.y * kcy + cam.dir.y,
                  cam.x.z * kcx + cam.y.z * kcy + cam.dir.z);
    st3(a.o, p, add3(smul3(0.1f, rdir), mk3(cam.orig.x, cam.orig.y, cam.orig.z)));
    st3(a.d, p, norm3(rdir));
    st3(a.rad, p, mk3(0.f, 0.f, 0.f));
    st3(a.tp, p, mk3(1.f, 1.f, 1.f));
}

// end of a pass (RadianceGPU's running mean, rendering_kernel.cl:1127-1136);
// returns true when the pixel starts another pass (its camera ray is written)
__device__ __forceinline__ bool wf_finish_pass(const WfArgs &a, int p, int4 &meta, uint32_t &s0,
                                               uint32_t &s1) {
    const f3 rad = ld3(a.rad, p);
    f3 col = ld3(a.col, p);
    const int cs = a.r.start_sample + meta.z;
    if (cs == 0) {
        col = rad;
    } else {
        const float k1 = (float)cs;
        const float k2 = 1.f / ((float)cs + 1.f);
        col.x = (col.x * k1 + rad.x) * k2;
        col.y = (col.y * k1 + rad.y) * k2;
        col.z = (col.z * k1 + rad.z) * k2;
    }
    st3(a.col, p, col);
    meta.z += 1;
    const int gid = meta.w;
    if (meta.z < a.r.passes) {
        wf_camera(a, p, gid, s0, s1);
        meta.x = 0;   // depth
        meta.y = 1;   // specularBounce
        return true;
    }
    const int x = gid % a.r.width, y = gid / a.r.width;
    ptgpu_vec out;
    out.x = col.x; out.y = col.y; out.z = col.z;
    a.r.colors[(a.r.height - y - 1) * a.r.width + x] = out;
    a.r.pixels[gid] = wf_to_int(col.x) | (wf_to_int(col.y) << 8) | (wf_to_int(col.z) << 16) |
                      0xff000000u;
    reinterpret_cast<uint2 *>(a.r.seeds)[gid] = make_uint2(s0, s1);
    return false;
}

}  // namespace

__global__ void __launch_bounds__(kWfThreads) k_wf_init(const WfArgs a, int base, int count) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= count) return;
    const int gid = base + p;
    const uint2 sd = reinterpret_cast<const uint2 *>(a.r.seeds)[gid];
    uint32_t s0 = sd.x, s1 = sd.y;
    f3 col = mk3(0.f, 0.f, 0.f);
    if (a.r.start_sample > 0) {
        const int x = gid % a.r.width, y = gid / a.r.width;
        const ptgpu_vec c = a.r.colors[(a.r.height - y - 1) * a.r.width + x];
        col = mk3(c.x, c.y, c.z);
    }
    st3(a.col, p, col);
    wf_camera(a, p, gid, s0, s1);
    a.seeds[p] = make_uint2(s0, s1);
    a.meta[p] = make_int4(0, 1, 0, gid);
    a.ext_in[p] = p;
    if (p == 0) a.counters[0] = (unsigned)count;
}

template <bool WIDE>
__global__ void __launch_bounds__(kWfThreads) k_wf_extend(const WfArgs a, const int *ext_in) {
    const unsigned n = a.counters[0];
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = ext_in[i];
        float t;
        int prim;
        const int h = trace_query<WIDE, false>(a.r.tv, ld3(a.o, p), ld3(a.d, p), false, 0.f, t, prim,
                                               nullptr);
        a.hit[p] = make_float2(t, __int_as_float(h ? prim : -2));
    }
}

template <bool WIDE>
__global__ void __launch_bounds__(kWfThreads) k_wf_shadow(const WfArgs a) {
    const unsigned n = a.counters[2];
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 so = a.sh_o[i], sdv = a.sh_d[i];
        float t;
        int prim;
        const int occ = trace_query<WIDE, false>(a.r.tv, mk3(so.x, so.y, so.z),
                                                 mk3(sdv.x, sdv.y, sdv.z), true, so.w, t, prim,
                                                 nullptr);
        a.sh_vis[i] = occ ? 0 : 1;
    }
}

__global__ void __launch_bounds__(kWfThreads) k_wf_shade(const WfArgs a, const int *ext_in,
                                                         int *ext_out) {
    const unsigned n = a.counters[0];
    const unsigned nround = (n + 31u) & ~31u;     // whole warps take part in the appends
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < nround;
         i += gridDim.x * blockDim.x) {
        const bool live = i < n;
        const int p = live ? ext_in[i] : 0;
        int next = 0;            // 0: nothing, 1: extension ray, 2: NEE pending
        int nsh = 0;
        float4 sho[kWfMaxLights], shd[kWfMaxLights], shc[kWfMaxLights];   // scenes with more lights use k_render
        int4 meta = make_int4(0, 0, 0, 0);
        uint2 sd = make_uint2(0, 0);
        if (live) {
            meta = a.meta[p];
            sd = a.seeds[p];
            uint32_t s0 = sd.x, s1 = sd.y;
            const float2 hit = a.hit[p];
            const int prim = __float_as_int(hit.y);
            bool finish = false;
            if (prim == -2) {
                finish = true;                       // miss: result = rad
            } else {
                const f3 o = ld3(a.o, p), d = ld3(a.d, p);
                const f3 hp = add3(o, smul3(hit.x, d));
                const int id = prim >= 0 ? __ldg(&a.r.tv.prim_id[prim]) : 0;
                const Material m = a.r.mats[id];
                const int type = __float_as_int(m.e_type.w);
                const float4 *pp = prim >= 0 ? a.r.tv.prims : a.r.prims0;
                const int k = prim >= 0 ? prim : 0;
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
                const f3 nl = smul3(inv_sign, normal);
                f3 ecol = mk3(m.e_type.x, m.e_type.y, m.e_type.z);
                const f3 colr = mk3(m.c_refl.x, m.c_refl.y, m.c_refl.z);
                const int refl = __float_as_int(m.c_refl.w);
                f3 tp = ld3(a.tp, p);
                if (!iszero3(ecol)) {
                    if (meta.y) {
                        ecol = smul3(fabsf(dp), ecol);
                        ecol = mul3(tp, ecol);
                        st3(a.rad, p, add3(ld3(a.rad, p), ecol));
                    }
                    finish = true;
                } else if (refl == PTGPU_DIFF) {
                    meta.y = 0;
                    tp = mul3(tp, colr);
                    st3(a.tp, p, tp);
                    // SampleLights: draw every light, keep the ones to test
                    for (int li = 0; li < a.r.n_lights; ++li) {
                        const LightRec L = a.r.lights[li];
                        float u1, u2;
                        if (a.r.rtl) { u2 = get_random(s0, s1); u1 = get_random(s0, s1); }
                        else         { u1 = get_random(s0, s1); u2 = get_random(s0, s1); }
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
                        f3 sdir = sub3(lp, hp);
                        const float len = sqrtf(dot3(sdir, sdir));
                        sdir = smul3(1.f / len, sdir);
                        float wo = dot3(sdir, lnrm);
                        if (wo > 0.f) continue;
                        wo = -wo;
                        wo = cl_clamp(wo, 0.f, 1.f);
                        const float wi = dot3(sdir, nl);
                        if (wi > 0.f && nsh < kWfMaxLights) {
                            const float s = L.b.w * wi * wo / (len * len);
                            const f3 c = smul3(s, mk3(L.e.x, L.e.y, L.e.z));
                            sho[nsh] = make_float4(hp.x, hp.y, hp.z, len - kEps);
                            shd[nsh] = make_float4(sdir.x, sdir.y, sdir.z, __int_as_float(p));
                            shc[nsh] = make_float4(c.x, c.y, c.z, 0.f);
                            ++nsh;
                        }
                    }
                    // the diffuse bounce
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
                    st3(a.o, p, hp);
                    st3(a.d, p, nd);
                    meta.x += 1;
                    if (nsh > 0) next = 2;
                    else if (meta.x > a.r.max_depth) finish = true;
                    else next = 1;
                } else if (refl == PTGPU_SPEC) {
                    meta.y = 1;
                    const f3 ndir = sub3(d, smul3(2.f * dot3(normal, d), normal));
                    st3(a.tp, p, mul3(tp, colr));
                    st3(a.o, p, hp);
                    st3(a.d, p, ndir);
                    meta.x += 1;
                    if (meta.x > a.r.max_depth) finish = true; else next = 1;
                } else {
                    meta.y = 1;
                    const f3 refl_d = sub3(d, smul3(2.f * dot3(normal, d), normal));
                    const bool into = dot3(normal, nl) > 0;
                    const float nc = 1.f, nt = 1.5f;
                    const float nnt = into ? nc / nt : nt / nc;
                    const float ddn = dot3(d, nl);
                    const float cos2t = 1.f - nnt * nnt * (1.f - ddn * ddn);
                    f3 ndir = refl_d;
                    if (cos2t < 0.f) {
                        tp = mul3(tp, colr);
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
                        } else {
                            tp = smul3(TP, tp);
                            tp = mul3(tp, colr);
                            ndir = tdir;
                        }
                    }
                    st3(a.tp, p, tp);
                    st3(a.o, p, hp);
                    st3(a.d, p, ndir);
                    meta.x += 1;
                    if (meta.x > a.r.max_depth) finish = true; else next = 1;
                }
            }
            if (finish) next = wf_finish_pass(a, p, meta, s0, s1) ? 1 : 0;
            sd = make_uint2(s0, s1);
            a.seeds[p] = sd;
        }
        // ---- compacted appends (whole warp)
        const int slot_e = wf_append1(&a.counters[1], live && next == 1);
        if (slot_e >= 0) ext_out[slot_e] = p;
        const int slot_p = wf_append1(&a.counters[3], live && next == 2);
        if (slot_p >= 0) a.pend[slot_p] = p;
        const int first = wf_appendn(&a.counters[2], (live && next == 2) ? nsh : 0);
        if (live && next == 2) {
            for (int k = 0; k < nsh; ++k) {
                a.sh_o[first + k] = sho[k];
                a.sh_d[first + k] = shd[k];
                a.sh_c[first + k] = shc[k];
            }
            a.nee[p] = make_int2(first, nsh);
        }
        if (live) a.meta[p] = meta;
    }
}

__global__ void __launch_bounds__(kWfThreads) k_wf_resolve(const WfArgs a, int *ext_out) {
    const unsigned n = a.counters[3];
    const unsigned nround = (n + 31u) & ~31u;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < nround;
         i += gridDim.x * blockDim.x) {
        const bool live = i < n;
        int p = 0, next = 0;
        if (live) {
            p = a.pend[i];
            const int2 ne = a.nee[p];
            f3 ld = mk3(0.f, 0.f, 0.f);
            for (int k = 0; k < ne.y; ++k)
                if (a.sh_vis[ne.x + k]) {
                    const float4 c = a.sh_c[ne.x + k];
                    ld = add3(ld, mk3(c.x, c.y, c.z));
                }
            ld = mul3(ld, ld3(a.tp, p));
            st3(a.rad, p, add3(ld3(a.rad, p), ld));
            int4 meta = a.meta[p];
            if (meta.x > a.r.max_depth) {
                uint2 sd = a.seeds[p];
                uint32_t s0 = sd.x, s1 = sd.y;
                next = wf_finish_pass(a, p, meta, s0, s1) ? 1 : 0;
                a.seeds[p] = make_uint2(s0, s1);
                a.meta[p] = meta;
            } else {
                next = 1;
            }
        }
        const int slot = wf_append1(&a.counters[1], live && next == 1);
        if (slot >= 0) ext_out[slot] = p;
    }
}

// next iteration: the extension queue just filled becomes the input
__global__ void k_wf_advance(unsigned *counters) {
    counters[0] = counters[1];
    counters[1] = 0;
    counters[2] = 0;
    counters[3] = 0;
}

void wf_carve(WfArgs &a, void *base, int paths, int n_lights) {
    const size_t P = (size_t)paths;
    const size_t L = (size_t)(n_lights < 1 ? 1 : (n_lights > 8 ? 8 : n_lights));
    char *q = static_cast<char *>(base);
    auto take = [&](size_t bytes) { void *r = q; q += (bytes + 255) & ~size_t(255); return r; };
    a.o = (float4 *)take(P * 16); a.d = (float4 *)take(P * 16); a.rad = (float4 *)take(P * 16);
    a.tp = (float4 *)take(P * 16); a.col = (float4 *)take(P * 16);
    a.seeds = (uint2 *)take(P * 8); a.meta = (int4 *)take(P * 16); a.nee = (int2 *)take(P * 8);
    a.hit = (float2 *)take(P * 8);
    a.ext_in = (int *)take(P * 4); a.ext_out = (int *)take(P * 4); a.pend = (int *)take(P * 4);
    a.sh_o = (float4 *)take(P * L * 16); a.sh_d = (float4 *)take(P * L * 16);
    a.sh_c = (float4 *)take(P * L * 16); a.sh_vis = (unsigned char *)take(P * L);
    a.counters = (unsigned *)take(64);
}

size_t wf_carve_bytes(int paths, int n_lights) {
    const size_t P = (size_t)paths;
    const size_t L = (size_t)(n_lights < 1 ? 1 : (n_lights > 8 ? 8 : n_lights));
    auto r = [](size_t b) { return (b + 255) & ~size_t(255); };
    return 5 * r(P * 16) + r(P * 8) + r(P * 16) + r(P * 8) + r(P * 8) + 3 * r(P * 4) +
           3 * r(P * L * 16) + r(P * L) + r(64);
}

cudaError_t launch_wavefront(WfArgs a, int iterations, int grid, cudaStream_t s) {
    const int npx = a.r.width * a.r.height;
    const bool wide = a.r.tv.nodes4 != nullptr;
    for (int base = 0; base < npx; base += a.paths) {
        const int count = npx - base < a.paths ? npx - base : a.paths;
        k_wf_init<<<(count + kWfThreads - 1) / kWfThreads, kWfThreads, 0, s>>>(a, base, count);
        cudaMemsetAsync(a.counters + 1, 0, 3 * sizeof(unsigned), s);
        int *qin = a.ext_in, *qout = a.ext_out;
        for (int it = 0; it < iterations; ++it) {
            if (wide) k_wf_extend<true><<<grid, kWfThreads, 0, s>>>(a, qin);
            else k_wf_extend<false><<<grid, kWfThreads, 0, s>>>(a, qin);
            k_wf_shade<<<grid, kWfThreads, 0, s>>>(a, qin, qout);
            if (wide) k_wf_shadow<true><<<grid, kWfThreads, 0, s>>>(a);
            else k_wf_shadow<false><<<grid, kWfThreads, 0, s>>>(a);
            k_wf_resolve<<<grid, kWfThreads, 0, s>>>(a, qout);
            k_wf_advance<<<1, 1, 0, s>>>(a.counters);
            int *t = qin; qin = qout; qout = t;
        }
    }
    return cudaGetLastError();
}

}  // namespace ptgpu
