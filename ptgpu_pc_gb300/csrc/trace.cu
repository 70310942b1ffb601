// trace.cu -- closest-hit queries and the per-pixel radiance path tracer.
//
// render: one thread per pixel runs all of the frame's passes back to back
// (RadianceGPU, rendering_kernel.cl:1072-1150, once per pass).  A pixel's
// passes are sequential by construction -- each pass continues the pixel's
// seed stream where the previous one left it -- so the pixel is the unit of
// parallelism; keeping its passes in one thread keeps the seeds, the running
// mean and the colour in registers for the whole frame and writes them once.
#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"
#include "lbvh.h"

namespace ptgpu {

__global__ void k_trace_closest(TraceView tv, const ptgpu_ray *__restrict__ rays, int n,
                                float *__restrict__ tout, uint32_t *__restrict__ idout,
                                int32_t *__restrict__ hitout) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *rp = reinterpret_cast<const float *>(rays + i);
    f3 o = mk3(rp[0], rp[1], rp[2]);
    f3 d = mk3(rp[3], rp[4], rp[5]);
    float t;
    int prim, id;
    int h = trace_closest(tv, o, d, t, prim, id);
    tout[i] = t;
    idout[i] = h ? (uint32_t)id : 0u;
    hitout[i] = h;
}

// SampleLights (rendering_kernel.cl:397-493) over the emitter list
template <bool COUNT>
__device__ __forceinline__ f3 sample_lights(const RenderArgs &a, uint32_t &s0, uint32_t &s1,
                                            f3 hit, f3 normal, Counts *cnt) {
    f3 result = mk3(0.f, 0.f, 0.f);
    for (int li = 0; li < a.n_lights; ++li) {
        const LightRec L = a.lights[li];
        f3 lp, ln;
        float u1, u2;
        if (a.rtl) { u2 = get_random(s0, s1); u1 = get_random(s0, s1); }
        else       { u1 = get_random(s0, s1); u2 = get_random(s0, s1); }
        if (__float_as_int(L.a.w) == PTGPU_TRIANGLE) {
            float su1 = sqrtf(u1);
            float bu = 1.0f - su1, bv = u2 * su1;
            f3 e1 = smul3(bu, mk3(L.b.x, L.b.y, L.b.z));
            f3 e2 = smul3(bv, mk3(L.c.x, L.c.y, L.c.z));
            lp = add3(add3(mk3(L.a.x, L.a.y, L.a.z), e1), e2);
            ln = norm3(cross3(e1, e2));
        } else {
            const float zz = 1.f - 2.f * u1;
            const float rr = sqrtf(fmaxf(0.f, 1.f - zz * zz));
            const float phi = 2.f * kPi * u2;
            float sphi, cphi;
            pt_sincos(phi, sphi, cphi);
            f3 unit = mk3(rr * cphi, rr * sphi, zz);
            lp = add3(smul3(L.b.x, unit), mk3(L.a.x, L.a.y, L.a.z));
            ln = unit;
        }
        f3 sd = sub3(lp, hit);
        const float len = sqrtf(dot3(sd, sd));
        sd = smul3(1.f / len, sd);
        float wo = dot3(sd, ln);
        if (wo > 0.f) continue;
        wo = -wo;
        wo = cl_clamp(wo, 0.f, 1.f);
        const float wi = dot3(sd, normal);
        if (COUNT && wi > 0.f) cnt[2].v++;   // shadow query issued
        if (wi > 0.f && !trace_any<COUNT>(a.tv, hit, sd, len - kEps, cnt + 1)) {
            const float s = L.b.w * wi * wo / (len * len);
            result = add3(result, smul3(s, mk3(L.e.x, L.e.y, L.e.z)));
        }
    }
    return result;
}

// RadiancePathTracing + RadianceOnePathTracing (rendering_kernel.cl:495-820)
template <bool COUNT>
__device__ __forceinline__ f3 radiance(const RenderArgs &a, f3 o, f3 d, uint32_t &s0,
                                       uint32_t &s1, Counts *cnt) {
    f3 rad = mk3(0.f, 0.f, 0.f);
    f3 tp = mk3(1.f, 1.f, 1.f);
    int specular = 1;
    for (int depth = 0; depth <= a.max_depth; ++depth) {
        float t;
        int prim, id;
        if (COUNT) cnt[2].p++;   // extension query issued
        if (!trace_closest<COUNT>(a.tv, o, d, t, prim, id, cnt)) break;
        f3 hp = add3(o, smul3(t, d));
        const Material m = a.mats[id];
        const int type = __float_as_int(m.e_type.w);
        f3 normal;
        {
            // geometry of the hit from the traversal-order prims; a hit
            // reported only beyond t = 1e20 keeps the reference's id = 0
            const int k = prim >= 0 ? prim : 0;
            const float4 *pp = prim >= 0 ? a.tv.prims : a.prims0;
            float4 g0 = __ldg(&pp[3 * k + 0]);
            if (type == PTGPU_SPHERE) {
                normal = sub3(hp, mk3(g0.x, g0.y, g0.z));
            } else {
                float4 g1 = __ldg(&pp[3 * k + 1]);
                float4 g2 = __ldg(&pp[3 * k + 2]);
                normal = cross3(mk3(g1.x, g1.y, g1.z), mk3(g2.x, g2.y, g2.z));
            }
        }
        normal = norm3(normal);
        const float dp = dot3(normal, d);
        const float inv_sign = -1.f * cl_sign(dp);
        f3 nl = smul3(inv_sign, normal);
        f3 ecol = mk3(m.e_type.x, m.e_type.y, m.e_type.z);
        if (!iszero3(ecol)) {
            if (specular) {
                ecol = smul3(fabsf(dp), ecol);
                ecol = mul3(tp, ecol);
                rad = add3(rad, ecol);
            }
            break;
        }
        f3 col = mk3(m.c_refl.x, m.c_refl.y, m.c_refl.z);
        const int refl = __float_as_int(m.c_refl.w);
        if (refl == PTGPU_DIFF) {
            specular = 0;
            tp = mul3(tp, col);
            f3 ld = sample_lights<COUNT>(a, s0, s1, hp, nl, cnt);
            ld = mul3(ld, tp);
            rad = add3(rad, ld);
            float r1 = 2.f * kPi * get_random(s0, s1);
            float r2 = get_random(s0, s1);
            float r2s = sqrtf(r2);
            f3 w = nl;
            f3 av = (fabsf(w.x) > .1f) ? mk3(0.f, 1.f, 0.f) : mk3(1.f, 0.f, 0.f);
            f3 u = norm3(cross3(av, w));
            f3 v = cross3(w, u);
            float sr1, cr1;
            pt_sincos(r1, sr1, cr1);
            u = smul3(cr1 * r2s, u);
            v = smul3(sr1 * r2s, v);
            f3 nd = add3(u, v);
            w = smul3(sqrtf(1.f - r2), w);
            nd = add3(nd, w);
            o = hp; d = nd;
        } else if (refl == PTGPU_SPEC) {
            specular = 1;
            f3 nd = sub3(d, smul3(2.f * dot3(normal, d), normal));
            tp = mul3(tp, col);
            o = hp; d = nd;
        } else {
            specular = 1;
            f3 refl_d = sub3(d, smul3(2.f * dot3(normal, d), normal));
            const bool into = dot3(normal, nl) > 0;
            const float nc = 1.f, nt = 1.5f;
            const float nnt = into ? nc / nt : nt / nc;
            const float ddn = dot3(d, nl);
            const float cos2t = 1.f - nnt * nnt * (1.f - ddn * ddn);
            if (cos2t < 0.f) {
                tp = mul3(tp, col);
                o = hp; d = refl_d;
                continue;
            }
            const float kk = (float)(into ? 1 : -1) * (ddn * nnt + sqrtf(cos2t));
            f3 nkk = smul3(kk, normal);
            f3 tdir = norm3(sub3(smul3(nnt, d), nkk));
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
                tp = mul3(tp, col);
                o = hp; d = refl_d;
            } else {
                tp = smul3(TP, tp);
                tp = mul3(tp, col);
                o = hp; d = tdir;
            }
        }
    }
    return rad;
}

__device__ __forceinline__ uint32_t to_int(float x) {
    return (uint32_t)(int)(powf(cl_clamp(x, 0.f, 1.f), 1.f / 2.2f) * 255.f + .5f);
}

// COUNT = true: the same kernel, also accumulating into a.stats[6]: extension
// node visits, prim tests; shadow node visits, prim tests; extension and
// shadow query counts.
template <bool COUNT>
__global__ void __launch_bounds__(128) k_render(const RenderArgs a) {
    Counts cnt[3] = {{0, 0}, {0, 0}, {0, 0}};
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = a.width, h = a.height;
    if (gid >= w * h) return;
    const int x = gid % w, y = gid / w;
    uint2 sd = reinterpret_cast<const uint2 *>(a.seeds)[gid];
    uint32_t s0 = sd.x, s1 = sd.y;
    const int ci = (h - y - 1) * w + x;
    f3 col = mk3(0.f, 0.f, 0.f);
    if (a.start_sample > 0) {
        const ptgpu_vec c = a.colors[ci];
        col = mk3(c.x, c.y, c.z);
    }
    const float inv_w = 1.f / (float)w, inv_h = 1.f / (float)h;
    const ptgpu_camera &cam = a.cam;
    for (int p = 0; p < a.passes; ++p) {
        const int cs = a.start_sample + p;
        // GenerateCameraRay (rendering_kernel.cl:1042-1070)
        const float r1 = get_random(s0, s1) - .5f;
        const float r2 = get_random(s0, s1) - .5f;
        const float kcx = ((float)x + r1) * inv_w - .5f;
        const float kcy = ((float)y + r2) * inv_h - .5f;
        f3 rdir = mk3(cam.x.x * kcx + cam.y.x * kcy + cam.dir.x,
                      cam.x.y * kcx + cam.y.y * kcy + cam.dir.y,
                      cam.x.z * kcx + cam.y.z * kcy + cam.dir.z);
        f3 rorig = add3(smul3(0.1f, rdir), mk3(cam.orig.x, cam.orig.y, cam.orig.z));
        rdir = norm3(rdir);
        f3 r = radiance<COUNT>(a, rorig, rdir, s0, s1, cnt);
        if (cs == 0) {
            col = r;
        } else {
            const float k1 = (float)cs;
            const float k2 = 1.f / ((float)cs + 1.f);
            col.x = (col.x * k1 + r.x) * k2;
            col.y = (col.y * k1 + r.y) * k2;
            col.z = (col.z * k1 + r.z) * k2;
        }
    }
    ptgpu_vec out;
    out.x = col.x; out.y = col.y; out.z = col.z;
    a.colors[ci] = out;
    a.pixels[gid] = to_int(col.x) | (to_int(col.y) << 8) | (to_int(col.z) << 16) | 0xff000000u;
    reinterpret_cast<uint2 *>(a.seeds)[gid] = make_uint2(s0, s1);
    if (COUNT) {
        atomicAdd(a.stats + 0, (unsigned long long)cnt[0].v);
        atomicAdd(a.stats + 1, (unsigned long long)cnt[0].p);
        atomicAdd(a.stats + 2, (unsigned long long)cnt[1].v);
        atomicAdd(a.stats + 3, (unsigned long long)cnt[1].p);
        atomicAdd(a.stats + 4, (unsigned long long)cnt[2].p);
        atomicAdd(a.stats + 5, (unsigned long long)cnt[2].v);
    }
}

cudaError_t launch_render(const RenderArgs &a, int block, cudaStream_t s) {
    const int n = a.width * a.height;
    if (n <= 0 || a.passes <= 0) return cudaSuccess;
    if (block <= 0) block = 128;
    if (a.stats) k_render<true><<<(n + block - 1) / block, block, 0, s>>>(a);
    else k_render<false><<<(n + block - 1) / block, block, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_trace_closest(const TraceView &tv, const ptgpu_ray *rays, int n, float *t,
                                 uint32_t *id, int32_t *hit, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_trace_closest<<<(n + 127) / 128, 128, 0, s>>>(tv, rays, n, t, id, hit);
    return cudaGetLastError();
}

}  // namespace ptgpu
