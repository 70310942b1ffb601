// lbvh.cu -- GPU LBVH build for the reference BVH layout (CLBVH + BVH.cl).
//
// Pipeline (reference mode, all on one stream):
//   k_centroid_bounds   centroid min/max over all shapes (CLBVH.cpp:91-123),
//                       and each shape's bound as an aligned 32-byte record
//   k_morton            30-bit Morton keys (CLBVH.cpp:125-164)
//   k_hist4             digit histograms of all four radix passes
//   k_onesweep x4       stable LSD radix sort of ~key (== the descending
//                       stable bubble sort, CLBVH.cpp:31-47), 8-bit digits,
//                       warp-level ranking through shared lane masks,
//                       decoupled look-back with a bounded spin
//   k_emit              per 256-leaf window: the leaf records, then every
//                       internal node inside the window, bounds by a
//                       warp-shuffle bottom-up reduction, then a climb over
//                       the windows for the nodes above them
//                       (kernelConstructRadixTree and kernelConstructBVHTree,
//                       BVH.cl:141-258, with the closed-form topology of
//                       lbvh_topo.cuh).  The batched build runs k_leaves
//                       (leaf records and the leaves' bounds in sorted order)
//                       and k_tiles_seg (1024-leaf tiles of every segment).
// The result is the reference's btn[N-1]/btl[N] arrays, resident on the
// device.  k_abi_to_trace then derives the 64-byte traversal nodes.
#include <cfloat>
#include <cstring>
#include <cstdint>
#include <mutex>
#include <cuda_runtime.h>

#include "device.cuh"
#include "lbvh.h"
#include "lbvh_topo.cuh"

namespace ptgpu {

// ---------------------------------------------------------------------------
// scene unpacking: AoS Shape (104 B) -> build vertices, prims, materials
// ---------------------------------------------------------------------------
__global__ void k_unpack_shapes(const ptgpu_shape *__restrict__ shapes, int n,
                                float *__restrict__ verts, uint8_t *__restrict__ type,
                                float4 *__restrict__ prims, Material *__restrict__ mats) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ptgpu_shape s = shapes[i];
    float *v = verts + 9 * (size_t)i;
    type[i] = (uint8_t)s.type;
    if (s.type == PTGPU_TRIANGLE) {
        const ptgpu_triangle &t = s.g.t;
        v[0] = t.p1.x; v[1] = t.p1.y; v[2] = t.p1.z;
        v[3] = t.p2.x; v[4] = t.p2.y; v[5] = t.p2.z;
        v[6] = t.p3.x; v[7] = t.p3.y; v[8] = t.p3.z;
        prims[3 * (size_t)i + 0] = make_float4(t.p1.x, t.p1.y, t.p1.z, __int_as_float(PTGPU_TRIANGLE));
        prims[3 * (size_t)i + 1] = make_float4(t.p2.x - t.p1.x, t.p2.y - t.p1.y, t.p2.z - t.p1.z, 0.f);
        prims[3 * (size_t)i + 2] = make_float4(t.p3.x - t.p1.x, t.p3.y - t.p1.y, t.p3.z - t.p1.z, 0.f);
    } else {
        const ptgpu_sphere &sp = s.g.s;
        v[0] = sp.p.x; v[1] = sp.p.y; v[2] = sp.p.z; v[3] = sp.rad;
        v[4] = v[5] = v[6] = v[7] = v[8] = 0.f;
        prims[3 * (size_t)i + 0] = make_float4(sp.p.x, sp.p.y, sp.p.z, __int_as_float(PTGPU_SPHERE));
        prims[3 * (size_t)i + 1] = make_float4(sp.rad * sp.rad, sp.rad, 0.f, 0.f);
        prims[3 * (size_t)i + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    Material m;
    m.c_refl = make_float4(s.c.x, s.c.y, s.c.z, __int_as_float(s.refl));
    m.e_type = make_float4(s.e.x, s.e.y, s.e.z, __int_as_float(s.type));
    mats[i] = m;
}

// bound of one shape (CLBVH::getBound, CLBVH.cpp:49-75) from the build vertices
__device__ __forceinline__ void shape_bound(const float *__restrict__ verts, int s, bool tri,
                                            float b[6]) {
    const float *v = verts + 9 * (size_t)s;
    if (tri) {
        float x1 = v[0], y1 = v[1], z1 = v[2], x2 = v[3], y2 = v[4], z2 = v[5];
        float x3 = v[6], y3 = v[7], z3 = v[8];
        b[0] = min2f(min2f(x1, x2), x3); b[1] = max2f(max2f(x1, x2), x3);
        b[2] = min2f(min2f(y1, y2), y3); b[3] = max2f(max2f(y1, y2), y3);
        b[4] = min2f(min2f(z1, z2), z3); b[5] = max2f(max2f(z1, z2), z3);
    } else {
        float px = v[0], py = v[1], pz = v[2], r = v[3];
        b[0] = px - r; b[1] = px + r;
        b[2] = py - r; b[3] = py + r;
        b[4] = pz - r; b[5] = pz + r;
    }
}

__device__ __forceinline__ f3 shape_centroid(const float *__restrict__ verts, int s, bool tri) {
    if (!tri) {
        const float *v = verts + 9 * (size_t)s;
        return mk3(v[0], v[1], v[2]);
    }
    float b[6];
    shape_bound(verts, s, true, b);
    return mk3((b[0] + b[1]) / 2.0f, (b[2] + b[3]) / 2.0f, (b[4] + b[5]) / 2.0f);
}

// order-preserving float <-> uint (for atomic min/max)
__device__ __forceinline__ uint32_t f2ord(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float ord2f(uint32_t u) {
    uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f; memcpy(&f, &b, 4); return f;
#endif
}

// Programmatic dependent launch between the build kernels: the next kernel
// is launched with programmatic stream serialisation and its CTAs wait for
// the previous kernel's completion and memory (griddepcontrol.wait) before
// they touch anything, which hides part of the launch gap (4M shapes:
// 0.457 -> 0.440 ms per build).  Letting dependents launch early as well
// (griddepcontrol.launch_dependents at kernel entry, PTGPU_PDL_TRIGGER=1)
// measured slower (0.496 ms): the waiting CTAs hold SM slots during the
// previous kernel's last wave.  In a kernel launched without the attribute
// the wait returns at once.
#ifndef PTGPU_PDL
#define PTGPU_PDL 1
#endif
#ifndef PTGPU_PDL_TRIGGER
#define PTGPU_PDL_TRIGGER 0
#endif
__device__ __forceinline__ void pdl_begin() {
#if PTGPU_PDL
#if PTGPU_PDL_TRIGGER
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}

__global__ void k_init_state(BuildState *st, uint32_t wait_limit) {
    int t = threadIdx.x;
    for (int i = t; i < 5 * 256; i += blockDim.x) (&st->hist[0][0])[i] = 0u;
    if (t < 5) st->tile_counter[t] = 0u;
    if (t == 0) {
        st->error = 0u;
        st->top_ticket = 0u;
        st->wait_limit = wait_limit;
        // the reference's initial values: FLT_MAX for minima, FLT_MIN for maxima
        for (int a = 0; a < 3; ++a) {
            st->cmin[a] = f2ord(FLT_MAX);
            st->cmax[a] = f2ord(FLT_MIN);
        }
    }
}

// The state block, the radix passes' look-back words and the emission's
// arrival counters of a single-tree build, cleared in one launch (block 0
// also writes the state's initial values).
__global__ void k_init_build(BuildState *st, uint4 *__restrict__ status, size_t status_quads,
                             uint32_t *__restrict__ arrivals, size_t arrival_words, uint32_t wait_limit) {
    if (blockIdx.x == 0) {
        const int t = threadIdx.x;
        for (int i = t; i < 5 * 256; i += blockDim.x) (&st->hist[0][0])[i] = 0u;
        if (t < 5) st->tile_counter[t] = 0u;
        if (t == 0) {
            st->error = 0u;
            st->top_ticket = 0u;
            st->wait_limit = wait_limit;
            for (int a = 0; a < 3; ++a) {   // the reference's FLT_MAX / FLT_MIN initial values
                st->cmin[a] = f2ord(FLT_MAX);
                st->cmax[a] = f2ord(FLT_MIN);
            }
        }
    }
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < status_quads; i += stride) status[i] = z;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < arrival_words; i += stride) arrivals[i] = 0u;
}

// ---------------------------------------------------------------------------
// L2 residency of the bound records.  k_emit gathers each leaf's 32-byte
// bound record in sorted order, i.e. at random; those records are written by
// k_centroid_bounds four radix passes earlier.  Data that only streams
// through L2 in between can be read and written with the streaming cache
// operator (.cs: evict first), so that the bound records are what L2 keeps
// until the gather.  PTGPU_L2_HINTS selects where, one bit per site:
//   1  the radix passes' key and value loads and stores
//   2  k_centroid_bounds' vertex copies
//   4  k_emit's index and bound-record loads (their last use)
//   8  k_emit's node-record stores
//  16  the bound records stored and re-read with an evict-last L2 policy
// ---------------------------------------------------------------------------
#ifndef PTGPU_L2_HINTS
#define PTGPU_L2_HINTS 0
#endif
constexpr int kL2Sort = 1, kL2Verts = 2, kL2Gather = 4, kL2Nodes = 8, kL2BoundsLast = 16;
__host__ __device__ constexpr bool l2_hint(int bit) { return (PTGPU_L2_HINTS & bit) != 0; }

template <int BIT> __device__ __forceinline__ uint32_t ld_hint_u32(const uint32_t *a) {
    if constexpr (l2_hint(BIT)) return __ldcs(a);
    else return __ldg(a);
}
template <int BIT> __device__ __forceinline__ int32_t ld_hint_s32(const int32_t *a) {
    if constexpr (l2_hint(BIT)) return __ldcs(a);
    else return __ldg(a);
}
template <int BIT> __device__ __forceinline__ float4 ld_hint_f4(const float4 *a) {
    if constexpr (l2_hint(BIT)) return __ldcs(a);
    else return __ldg(a);
}
template <int BIT> __device__ __forceinline__ void st_hint_u32(uint32_t *a, uint32_t v) {
    if constexpr (l2_hint(BIT)) __stcs(a, v);
    else *a = v;
}
template <int BIT> __device__ __forceinline__ void st_hint_u4(uint4 *a, uint4 v) {
    if constexpr (l2_hint(BIT)) __stcs(a, v);
    else *a = v;
}
// evict-last L2 policy accesses of the bound records (bit 16)
__device__ __forceinline__ void st_last_f4(float4 *a, float4 v) {
    asm volatile("{\n\t.reg .b64 pol;\n\t"
                 "createpolicy.fractional.L2::evict_last.b64 pol, 1.0;\n\t"
                 "st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, pol;\n\t}" ::"l"(a),
                 "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}
__device__ __forceinline__ float4 ld_last_f4(const float4 *a) {
    float4 v;
    asm("{\n\t.reg .b64 pol;\n\t"
        "createpolicy.fractional.L2::evict_last.b64 pol, 1.0;\n\t"
        "ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], pol;\n\t}"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(a));
    return v;
}

// Centroid bounds, and each shape's bound stored as one aligned 32-byte
// record for the later kernels (the emission kernel gathers it in sorted
// order: one sector per leaf instead of a 36-byte vertex triple).
// one shape's bound, its 32-byte record and its share of the centroid bounds
__device__ __forceinline__ void centroid_shape(const float *__restrict__ v, bool tri,
                                               float4 *__restrict__ rec, float lo[3], float hi[3]) {
    float b[6];
    shape_bound(v, 0, tri, b);
    if constexpr (l2_hint(kL2BoundsLast)) {
        st_last_f4(rec, make_float4(b[0], b[1], b[2], b[3]));
        st_last_f4(rec + 1, make_float4(b[4], b[5], 0.f, 0.f));
    } else {
        rec[0] = make_float4(b[0], b[1], b[2], b[3]);
        rec[1] = make_float4(b[4], b[5], 0.f, 0.f);
    }
    const float c[3] = {tri ? (b[0] + b[1]) / 2.0f : v[0], tri ? (b[2] + b[3]) / 2.0f : v[1],
                        tri ? (b[4] + b[5]) / 2.0f : v[2]};
    for (int a = 0; a < 3; ++a) {
        if (c[a] == c[a]) {          // NaN centroids never pass the reference's < / >
            lo[a] = fminf(lo[a], c[a]);
            hi[a] = fmaxf(hi[a], c[a]);
        }
    }
}

#ifndef PTGPU_CENTROID_PIPE
#define PTGPU_CENTROID_PIPE 1
#endif

// 16-byte global -> shared copies that complete asynchronously (L2 only)
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
    if constexpr (l2_hint(kL2Verts)) {   // vertices are read once: evict first
        asm volatile("{\n\t.reg .b64 pol;\n\t"
                     "createpolicy.fractional.L2::evict_first.b64 pol, 1.0;\n\t"
                     "cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, pol;\n\t}" ::"r"(d),
                     "l"(gmem_src)
                     : "memory");
    } else {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem_src) : "memory");
    }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// A warp takes 32 consecutive shapes per step: their 1152 bytes of vertices
// arrive as 72 coalesced 16-byte loads (vertex array on a 16-byte boundary),
// go through shared memory, and each lane reads back its own 9 floats
// (stride 9: no bank conflicts).  The tail, or an unaligned array, takes one
// shape per lane directly.
__global__ void __launch_bounds__(256) k_centroid_bounds(const float *__restrict__ verts,
                                                          const uint8_t *__restrict__ type,
                                                          int all_tri, int n, BuildState *st,
                                                          float4 *__restrict__ aabbs) {
    pdl_begin();
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const bool aligned = (reinterpret_cast<uintptr_t>(verts) & 15) == 0;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
#if PTGPU_CENTROID_PIPE
    // two buffers per warp: the next 32 shapes' vertices are copied in
    // (cp.async, 16 bytes per copy) while the current ones are bounded
    __shared__ __align__(16) float s_v[256 / 32][2][32 * 9];
    const int stride = nwarps * 32;
    auto fetch = [&](int b, int slot) {
        if (aligned && b + 32 <= n) {
            const float4 *src = reinterpret_cast<const float4 *>(verts + 9 * (size_t)b);
            float4 *dst = reinterpret_cast<float4 *>(s_v[w][slot]);
            cp_async16(dst + lane, src + lane);
            cp_async16(dst + lane + 32, src + lane + 32);
            if (lane < 8) cp_async16(dst + lane + 64, src + lane + 64);
        }
        cp_async_commit();                        // one group per step, empty or not
    };
    int base = (blockIdx.x * (blockDim.x >> 5) + w) * 32;
    fetch(base, 0);
    for (int it = 0; base < n; ++it, base += stride) {
        fetch(base + stride, (it + 1) & 1);
        cp_async_wait1();                         // this step's copies have landed
        __syncwarp();
        const int i = base + lane;
        if (aligned && base + 32 <= n) {
            centroid_shape(s_v[w][it & 1] + 9 * lane, all_tri || type[i] == PTGPU_TRIANGLE, aabbs + 2 * (size_t)i,
                           lo, hi);
        } else if (i < n) {
            centroid_shape(verts + 9 * (size_t)i, all_tri || type[i] == PTGPU_TRIANGLE, aabbs + 2 * (size_t)i, lo, hi);
        }
        __syncwarp();                             // the buffer is read before it is refilled
    }
    cp_async_wait0();
#else
    __shared__ __align__(16) float s_v[256 / 32][32 * 9];
    float *sv = s_v[w];
    for (int base = (blockIdx.x * (blockDim.x >> 5) + w) * 32; base < n; base += nwarps * 32) {
        const int i = base + lane;
        if (aligned && base + 32 <= n) {
            const float4 *src = reinterpret_cast<const float4 *>(verts + 9 * (size_t)base);
            float4 *dst = reinterpret_cast<float4 *>(sv);
            dst[lane] = __ldg(src + lane);
            dst[lane + 32] = __ldg(src + lane + 32);
            if (lane < 8) dst[lane + 64] = __ldg(src + lane + 64);
            __syncwarp();
            centroid_shape(sv + 9 * lane, all_tri || type[i] == PTGPU_TRIANGLE, aabbs + 2 * (size_t)i, lo, hi);
            __syncwarp();
        } else if (i < n) {
            centroid_shape(verts + 9 * (size_t)i, all_tri || type[i] == PTGPU_TRIANGLE, aabbs + 2 * (size_t)i, lo, hi);
        }
    }
#endif
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    __shared__ float s_lo[8][3], s_hi[8][3];
    if (lane == 0) for (int a = 0; a < 3; ++a) { s_lo[w][a] = lo[a]; s_hi[w][a] = hi[a]; }
    __syncthreads();
    if (threadIdx.x < 3) {
        int a = threadIdx.x;
        float x = s_lo[0][a], y = s_hi[0][a];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { x = fminf(x, s_lo[k][a]); y = fmaxf(y, s_hi[k][a]); }
        if (x <= y || x == FLT_MAX) {
            atomicMin(&st->cmin[a], f2ord(x));
            atomicMax(&st->cmax[a], f2ord(y));
        }
    }
}

__device__ __forceinline__ uint32_t quantise10(float p, float lo, float hi) {
    float q = ((p - lo) / (hi - lo)) * 1024.f;
    if (!(q >= 0.f)) return 0u;          // NaN (hi == lo) is defined as 0
    if (q >= 4294967296.f) return 0u;
    return __float2uint_rz(q);
}

// bit j of a 10-bit value to bit 3j, by shift-and-mask steps that spread
// the bits apart (the same result as moving each bit separately)
__host__ __device__ __forceinline__ uint32_t spread3(uint32_t x) {
    x &= 1023u;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__host__ __device__ __forceinline__ uint32_t morton30(uint32_t a, uint32_t b, uint32_t c) {
    // bit j of a (j = 9..0) goes to 3j+2, of b to 3j+1, of c to 3j (CLBVH.cpp:158-163)
    return (spread3(a) << 2) | (spread3(b) << 1) | spread3(c);
}

// One warp's keys into the per-CTA digit counts of the four radix passes; a
// digit that every valid lane shares (spatially coherent keys) costs one
// atomic.
__device__ __forceinline__ void count_digits(uint32_t *s_hist, uint32_t key, bool valid, int lane) {
    const unsigned vm = __ballot_sync(0xffffffffu, valid);
    if (!vm) return;                        // lane 0 is valid when any lane is
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        const uint32_t dg = (key >> (8 * d)) & 255u;
        const uint32_t d0 = __shfl_sync(0xffffffffu, dg, 0);
        if (__all_sync(0xffffffffu, !valid || dg == d0)) {
            if (lane == 0) atomicAdd(&s_hist[d * 256 + d0], (uint32_t)__popc(vm));
        } else if (valid) {
            atomicAdd(&s_hist[d * 256 + dg], 1u);
        }
    }
}

// Morton keys.  The sort key is ~code, so an ascending stable sort gives the
// reference's descending stable order.  Blocks walk the shapes from the end
// back to the start: the tail of the array, read last by k_centroid_bounds,
// is still in L2 when this kernel starts.  Each thread loads its next step's
// record before it makes the current key.
// HIST: the digit histograms of the four radix passes are counted here as
// well (per-CTA shared counters, flushed once per CTA), so no separate
// histogram kernel re-reads the keys; a digit that every valid lane of the
// warp shares (spatially coherent keys) costs one atomic.
template <bool HIST>
__global__ void __launch_bounds__(256) k_morton(const float *__restrict__ verts,
                                                 const float4 *__restrict__ aabbs,
                                                 const uint8_t *__restrict__ type, int all_tri,
                                                 int n, BuildState *st,
                                                 uint32_t *__restrict__ keys) {
    pdl_begin();
    __shared__ uint32_t s_hist[HIST ? 4 * 256 : 1];
    if (HIST) {
        for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) s_hist[i] = 0u;
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) { lo[a] = ord2f(st->cmin[a]); hi[a] = ord2f(st->cmax[a]); }
    const int nblocks = (n + 255) / 256;
    // the next step's records are loaded before this step's keys are made
    // (a triangle's bound record; a sphere's centre in r0.xyz)
    auto fetch = [&](int blk, float4 &r0, float4 &r1, bool &tri) {
        const int i = blk * 256 + threadIdx.x;
        r0 = r1 = make_float4(0.f, 0.f, 0.f, 0.f);
        tri = true;
        if (blk >= 0 && i < n) {
            tri = all_tri || type[i] == PTGPU_TRIANGLE;
            if (tri) {
                if constexpr (l2_hint(kL2BoundsLast)) {   // read again by k_emit: keep
                    r0 = ld_last_f4(aabbs + 2 * (size_t)i);
                    r1 = ld_last_f4(aabbs + 2 * (size_t)i + 1);
                } else {
                    r0 = aabbs[2 * (size_t)i];
                    r1 = aabbs[2 * (size_t)i + 1];
                }
            } else {
                const f3 c = shape_centroid(verts, i, false);
                r0 = make_float4(c.x, c.y, c.z, 0.f);
            }
        }
    };
    float4 c0, c1;
    bool ctri;
    fetch(nblocks - 1 - (int)blockIdx.x, c0, c1, ctri);
    for (int blk = nblocks - 1 - (int)blockIdx.x; blk >= 0; blk -= gridDim.x) {
        float4 n0, n1;
        bool ntri;
        fetch(blk - (int)gridDim.x, n0, n1, ntri);
        const int i = blk * 256 + threadIdx.x;
        const bool valid = i < n;
        uint32_t key = 0;
        if (valid) {
            f3 p;
            if (ctri)    // the triangle's centroid is its bound's centre
                p = mk3((c0.x + c0.y) / 2.0f, (c0.z + c0.w) / 2.0f, (c1.x + c1.y) / 2.0f);
            else
                p = mk3(c0.x, c0.y, c0.z);
            uint32_t qa = quantise10(p.x, lo[0], hi[0]);
            uint32_t qb = quantise10(p.y, lo[1], hi[1]);
            uint32_t qc = quantise10(p.z, lo[2], hi[2]);
            key = ~morton30(qa & 1023u, qb & 1023u, qc & 1023u);
            keys[i] = key;
        }
        if (HIST) count_digits(s_hist, key, valid, lane);
        c0 = n0;
        c1 = n1;
        ctri = ntri;
    }
    if (HIST) {
        __syncthreads();
        for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x)
            if (s_hist[i]) atomicAdd(&st->hist[0][0] + i, s_hist[i]);
    }
}

// Digit histograms of all four passes.  Each thread counts runs of equal
// digits over 16 consecutive keys before touching shared memory, so the
// long runs of spatially coherent keys cost one atomic each.
constexpr int kHistItems = 16;
__global__ void __launch_bounds__(256) k_hist4(const uint32_t *__restrict__ keys, int n,
                                                BuildState *st) {
    pdl_begin();
    __shared__ uint32_t s_hist[4][256];
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0u;
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x * kHistItems;
    for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kHistItems; base < n;
         base += stride) {
        uint32_t k[kHistItems];
        if (base + kHistItems <= n) {
            const uint4 *p = reinterpret_cast<const uint4 *>(keys + base);
#pragma unroll
            for (int q = 0; q < kHistItems / 4; ++q) {
                uint4 v = p[q];
                k[4 * q] = v.x; k[4 * q + 1] = v.y; k[4 * q + 2] = v.z; k[4 * q + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int q = 0; q < kHistItems; ++q) k[q] = base + q < n ? keys[base + q] : 0u;
        }
        const int cnt = (int)min((int64_t)kHistItems, (int64_t)n - base);
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            uint32_t cur = (k[0] >> (8 * d)) & 255u, run = 1;
#pragma unroll
            for (int q = 1; q < kHistItems; ++q) {
                if (q >= cnt) break;
                uint32_t dg = (k[q] >> (8 * d)) & 255u;
                if (dg == cur) { ++run; continue; }
                atomicAdd(&s_hist[d][cur], run);
                cur = dg;
                run = 1;
            }
            atomicAdd(&s_hist[d][cur], run);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) {
        uint32_t v = (&s_hist[0][0])[i];
        if (v) atomicAdd(&st->hist[0][0] + i, v);
    }
}

// the segment holding shape v: the last s with off[s] <= v
__device__ __forceinline__ uint32_t segment_of(const int32_t *off, int n_segs, int32_t v) {
    int lo = 0, hi = n_segs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= v) lo = mid; else hi = mid - 1;
    }
    return (uint32_t)lo;
}

// ---------------------------------------------------------------------------
// segmented build: per-segment centroid bounds and Morton keys
// ---------------------------------------------------------------------------
__global__ void k_seg_init(SegState *ss, int n_segs, BuildState *st, const int32_t *seg_off) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_segs) return;
    for (int a = 0; a < 3; ++a) {
        ss[g].cmin[a] = f2ord(FLT_MAX);
        ss[g].cmax[a] = f2ord(FLT_MIN);
    }
    // the segment pass counts every shape of a segment under its digit
    st->hist[4][g] = (uint32_t)(seg_off[g + 1] - seg_off[g]);
}

// Same per-shape work as k_centroid_bounds; the min/max go to the shape's
// segment (one set of atomics per warp when the warp lies in one segment).
__global__ void __launch_bounds__(256) k_seg_centroid_bounds(const float *__restrict__ verts,
                                                              const uint8_t *__restrict__ type,
                                                              int n, SegBuild sb,
                                                              float4 *__restrict__ aabbs) {
    __shared__ int32_t s_off[kMaxSegments + 1];
    for (int i = threadIdx.x; i <= sb.n_segs; i += blockDim.x) s_off[i] = sb.seg_off[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t start = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    // every lane of a warp runs the same number of rounds
    const int64_t rounds = ((int64_t)n + stride - 1) / stride;
    for (int64_t r = 0; r < rounds; ++r) {
        const int64_t i = start + r * stride;
        const bool valid = i < n;
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        int g = 0;
        if (valid) {
            g = (int)segment_of(s_off, sb.n_segs, (int32_t)i);
            const bool tri = type[i] == PTGPU_TRIANGLE;
            float b[6];
            shape_bound(verts, (int)i, tri, b);
            aabbs[2 * i] = make_float4(b[0], b[1], b[2], b[3]);
            aabbs[2 * i + 1] = make_float4(b[4], b[5], 0.f, 0.f);
            const f3 p = tri ? mk3((b[0] + b[1]) / 2.0f, (b[2] + b[3]) / 2.0f, (b[4] + b[5]) / 2.0f)
                             : shape_centroid(verts, (int)i, false);
            const float c[3] = {p.x, p.y, p.z};
            for (int a = 0; a < 3; ++a)
                if (c[a] == c[a]) { lo[a] = c[a]; hi[a] = c[a]; }   // NaN never counts
        }
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
        const int g0 = __shfl_sync(0xffffffffu, g, __ffs(vm | 1u) - 1);
        const bool one = __all_sync(0xffffffffu, !valid || g == g0);
        if (one) {
            for (int a = 0; a < 3; ++a) {
                for (int o = 16; o > 0; o >>= 1) {
                    lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
                    hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
                }
            }
            if (lane == 0 && vm) {
                for (int a = 0; a < 3; ++a) {
                    if (lo[a] <= hi[a]) {
                        atomicMin(&sb.seg_state[g0].cmin[a], f2ord(lo[a]));
                        atomicMax(&sb.seg_state[g0].cmax[a], f2ord(hi[a]));
                    }
                }
            }
        } else if (valid) {
            for (int a = 0; a < 3; ++a) {
                if (lo[a] <= hi[a]) {
                    atomicMin(&sb.seg_state[g].cmin[a], f2ord(lo[a]));
                    atomicMax(&sb.seg_state[g].cmax[a], f2ord(hi[a]));
                }
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_seg_morton(const float *__restrict__ verts,
                                                     const float4 *__restrict__ aabbs,
                                                     const uint8_t *__restrict__ type, int n,
                                                     SegBuild sb, uint32_t *__restrict__ keys) {
    __shared__ int32_t s_off[kMaxSegments + 1];
    for (int i = threadIdx.x; i <= sb.n_segs; i += blockDim.x) s_off[i] = sb.seg_off[i];
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)segment_of(s_off, sb.n_segs, (int32_t)i);
        float lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = ord2f(__ldg(&sb.seg_state[g].cmin[a]));
            hi[a] = ord2f(__ldg(&sb.seg_state[g].cmax[a]));
        }
        const bool tri = type[i] == PTGPU_TRIANGLE;
        f3 p;
        if (tri) {
            const float4 b0 = aabbs[2 * i], b1 = aabbs[2 * i + 1];
            p = mk3((b0.x + b0.y) / 2.0f, (b0.z + b0.w) / 2.0f, (b1.x + b1.y) / 2.0f);
        } else {
            p = shape_centroid(verts, (int)i, false);
        }
        const uint32_t qa = quantise10(p.x, lo[0], hi[0]);
        const uint32_t qb = quantise10(p.y, lo[1], hi[1]);
        const uint32_t qc = quantise10(p.z, lo[2], hi[2]);
        keys[i] = ~morton30(qa & 1023u, qb & 1023u, qc & 1023u);
    }
}

// ---------------------------------------------------------------------------
// onesweep radix pass
// ---------------------------------------------------------------------------
#ifndef PTGPU_SORT_THREADS
#define PTGPU_SORT_THREADS 256
#endif
constexpr int kSortThreads = PTGPU_SORT_THREADS;   // 256 or 512; threads 0-255 own one digit each
static_assert(kSortThreads == 256 || kSortThreads == 512, "one digit per thread of the first 256");
constexpr int kSortWarps = kSortThreads / 32;
#ifndef PTGPU_SORT_ITEMS
#define PTGPU_SORT_ITEMS 20
#endif
constexpr int kSortItems = PTGPU_SORT_ITEMS;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr uint32_t kFlagAgg = 1u << 30, kFlagInc = 2u << 30, kValMask = (1u << 30) - 1u;
#ifndef PTGPU_LOOKBACK
#define PTGPU_LOOKBACK 8
#endif
constexpr int kLookback = PTGPU_LOOKBACK;   // predecessors read per look-back step
#ifndef PTGPU_SORT_PREFETCH
#define PTGPU_SORT_PREFETCH 1
#endif
#ifndef PTGPU_SORT_MINBLOCKS
#define PTGPU_SORT_MINBLOCKS 3
#endif
#ifndef PTGPU_SKIP_EMPTY_DIGITS
#define PTGPU_SKIP_EMPTY_DIGITS 1
#endif

// Look-back words are read and published with relaxed GPU-scope accesses:
// each read sees the word as it is in L2, and several reads of one thread
// can be in flight at once.
__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// block-wide exclusive scan of one value per thread (256 threads)
__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t v, uint32_t *s_tmp) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_tmp[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = lane < kSortWarps ? s_tmp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kSortWarps) s_tmp[lane] = t;
    }
    __syncthreads();
    uint32_t warp_base = w ? s_tmp[w - 1] : 0u;
    __syncthreads();
    return warp_base + x - v;
}

// Decoupled look-back of one digit (one thread per digit): publishes the
// tile's count as an aggregate (tile 0: as inclusive), sums predecessors back
// to the first inclusive word and publishes the inclusive count.  Returns the
// count of this digit in all earlier tiles.  A tile that has waited
// st->wait_limit times (kDefaultWaitLimit unless the caller lowered it; 0
// gives up before the first read) sets the build's error bit and its abort
// flag: it then scatters nothing, and every later kernel stays in bounds
// (destinations are checked against n, gathered indices clamped to [0, n)).
__device__ __forceinline__ uint32_t lookback_digit(uint32_t *status, int tile, int tid, uint32_t count,
                                                   BuildState *st, int &abort_flag) {
    uint32_t *my = status + (size_t)tile * 256 + tid;
    uint32_t excl = 0;
    if (tile == 0) {
        st_volatile(my, kFlagInc | count);
        return 0u;
    }
    st_volatile(my, kFlagAgg | count);
    // the words of kLookback predecessors are read at once, then summed from
    // the nearest back to the first inclusive one; a word not yet published
    // ends the window and is read again
    int p = tile - 1;
    bool timed_out = false;
    const uint32_t limit = st->wait_limit;
    uint32_t spins = 0;
    while (p >= 0) {
        if (spins >= limit) { timed_out = true; break; }
        uint32_t v[kLookback];
#pragma unroll
        for (int q = 0; q < kLookback; ++q)
            v[q] = p - q >= 0 ? ld_volatile(status + (size_t)(p - q) * 256 + tid) : 0u;
        int q = 0;
        bool done = false;
#pragma unroll
        for (; q < kLookback; ++q) {
            const uint32_t f = v[q] & (3u << 30);
            if (f == 0u) break;
            excl += v[q] & kValMask;
            if (f == kFlagInc) { done = true; break; }
        }
        if (done) break;
        p -= q;
        if (q < kLookback) {
            ++spins;
            __nanosleep(32);
        }
    }
    if (timed_out) { atomicOr(&st->error, 1u); abort_flag = 1; }
    st_volatile(my, kFlagInc | ((excl + count) & kValMask));
    return excl;
}

// Ranking chains per warp: with 2, a warp's items are ranked as two
// independent runs (the first and the second half of its items), each with
// its own per-digit counts, interleaved item by item, so that one run's
// shared-memory round trips (lane mask, count load, count store) overlap the
// other's; the second run's ranks are then offset by the first run's counts.
// Measured at 4M keys: 0.369 ms per build with 2 against 0.364 with 1 (the
// extra shared memory and the rank fix-up cost more than the overlap gains).
#ifndef PTGPU_SORT_CHAINS
#define PTGPU_SORT_CHAINS 1
#endif
constexpr int kSortChains = PTGPU_SORT_CHAINS;
static_assert(kSortChains == 1 || kSortChains == 2, "one or two ranking chains");
constexpr int kChainItems = (kSortItems + kSortChains - 1) / kSortChains;

struct SortSmem {
    uint32_t warp_hist[kSortWarps][256];          // the first chain's counts, then the warp's
    uint32_t chain_hist[kSortWarps][kSortChains > 1 ? 256 : 4];   // the second chain's counts
    uint32_t digit_start[256];
    uint32_t tile_excl[256];
    uint32_t scan_tmp[32];
    union {
        // ranking: per-warp lane masks of each digit and chain, two sets used
        // by alternate items so that clearing one never races with filling it
        uint32_t match[2][kSortChains][kSortWarps][256];
        // scatter: the tile in sorted order
        struct {
            uint32_t keys[kSortTile];
            int32_t vals[kSortTile];
        } st;
    } u;
    int32_t seg_off[kMaxSegments + 1];   // SEG: the segments' first shapes
    int tile;
    int abort;
};

// One pass: stable counting sort of (key, val) by the 8-bit digit of key at
// 8 * pass.  SEG (the last pass of a segmented build): the digit is the
// segment of the value (a shape id), so the pass regroups the shapes by
// segment and keeps each segment's key order.
template <bool FIRST, bool LAST, bool SEG = false>
__global__ void __launch_bounds__(kSortThreads, PTGPU_SORT_MINBLOCKS) k_onesweep(const uint32_t *__restrict__ keys_in,
                                                            const int32_t *__restrict__ vals_in,
                                                            uint32_t *__restrict__ keys_out,
                                                            int32_t *__restrict__ vals_out, int n,
                                                            int pass, BuildState *st,
                                                            uint32_t *status,
                                                            const int32_t *__restrict__ seg_off = nullptr,
                                                            int n_segs = 0) {
    pdl_begin();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem &sm = *reinterpret_cast<SortSmem *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int shift = SEG ? 0 : 8 * pass;
    if (tid == 0) { sm.tile = (int)atomicAdd(&st->tile_counter[pass], 1u); sm.abort = 0; }
    if (SEG)
        for (int i = tid; i <= n_segs; i += kSortThreads) sm.seg_off[i] = seg_off[i];
    static_assert(kSortWarps * 256 % (4 * kSortThreads) == 0, "16-byte clears");
    const uint4 zero4 = make_uint4(0u, 0u, 0u, 0u);
    for (int i = tid; i < kSortWarps * 64; i += kSortThreads) reinterpret_cast<uint4 *>(&sm.warp_hist[0][0])[i] = zero4;
    if (kSortChains > 1)
        for (int i = tid; i < kSortWarps * 64; i += kSortThreads)
            reinterpret_cast<uint4 *>(&sm.chain_hist[0][0])[i] = zero4;
    for (int i = tid; i < 2 * kSortChains * kSortWarps * 64; i += kSortThreads)
        reinterpret_cast<uint4 *>(&sm.u.match[0][0][0][0])[i] = zero4;
    // global digit offsets for this pass
    const bool dig_thread = kSortThreads == 256 || tid < 256;
    uint32_t gcount = dig_thread ? st->hist[pass][tid] : 0u;
#if PTGPU_SORT_PREFETCH
    __syncthreads();                          // the tile id, seg_off, the cleared arrays
    uint32_t goff = 0;
#else
    uint32_t goff = block_excl_scan256(gcount, sm.scan_tmp);
    __syncthreads();
#endif
    const int tile = sm.tile;
    // 64-bit positions: measured faster here than 32-bit ones (4M keys: 4 passes
    // 0.148 -> 0.183 ms with int)
    const int64_t base = (int64_t)tile * kSortTile;
    // the values are read again when they are staged (from L2), so that the
    // registers they would hold go to more items per tile
    uint32_t key[kSortItems];
    uint32_t rank[kSortItems];
    const unsigned lt_mask = (1u << lane) - 1u;
    // all loads first: the ranking below synchronises the warp per item, and
    // a load may not move across that
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const int64_t idx = base + (int64_t)w * 32 * kSortItems + j * 32 + lane;
        const bool valid = idx < n;
        if constexpr (SEG) {   // seg_off is in shared memory after the barrier above
            const int32_t v = valid ? ld_hint_s32<kL2Sort>(vals_in + idx) : -1;
            key[j] = v >= 0 ? segment_of(sm.seg_off, n_segs, v) : 0xffffffffu;
        } else {
            key[j] = valid ? ld_hint_u32<kL2Sort>(keys_in + idx) : 0xffffffffu;
        }
    }
#if PTGPU_SORT_PREFETCH
    // the scan of the global digit counts runs while the tile's loads are in flight
    goff = block_excl_scan256(gcount, sm.scan_tmp);
#endif
#pragma unroll
    for (int k = 0; k < kChainItems; ++k) {
        // item k of every chain: lanes with the same digit each set their bit
        // in the digit's mask
        uint32_t *mask[kSortChains];
        uint32_t dig[kSortChains];
        bool valid[kSortChains];
#pragma unroll
        for (int c = 0; c < kSortChains; ++c) {
            const int j = c * kChainItems + k;
            valid[c] = false;
            if (j < kSortItems) {
                const int64_t idx = base + (int64_t)w * 32 * kSortItems + j * 32 + lane;
                valid[c] = idx < n;
                dig[c] = (key[j] >> shift) & 255u;
                mask[c] = &sm.u.match[k & 1][c][w][dig[c]];
                if (valid[c]) atomicOr(mask[c], 1u << lane);
            }
        }
        __syncwarp();
        uint32_t prev[kSortChains];
        unsigned peers[kSortChains];
#pragma unroll
        for (int c = 0; c < kSortChains; ++c) {
            const int j = c * kChainItems + k;
            if (j >= kSortItems) continue;
            rank[j] = 0xffffffffu;
            prev[c] = 0u;
            peers[c] = 0u;
            if (valid[c]) {
                uint32_t *hist = c == 0 ? &sm.warp_hist[w][0] : &sm.chain_hist[w][0];
                peers[c] = *mask[c];
                prev[c] = hist[dig[c]];
                rank[j] = prev[c] + (uint32_t)__popc(peers[c] & lt_mask);
            }
        }
        __syncwarp();
#pragma unroll
        for (int c = 0; c < kSortChains; ++c) {
            const int j = c * kChainItems + k;
            if (j < kSortItems && valid[c] && lane == __ffs(peers[c]) - 1) {
                uint32_t *hist = c == 0 ? &sm.warp_hist[w][0] : &sm.chain_hist[w][0];
                hist[dig[c]] = prev[c] + (uint32_t)__popc(peers[c]);
                *mask[c] = 0u;
            }
        }
    }
    if (kSortChains > 1) {
        // the second chain's items follow the first chain's in the warp's
        // order: offset their ranks by the first chain's counts, then make
        // warp_hist the warp's totals
        __syncwarp();
#pragma unroll
        for (int j = kChainItems; j < kSortItems; ++j)
            if (rank[j] != 0xffffffffu) rank[j] += sm.warp_hist[w][(key[j] >> shift) & 255u];
        __syncwarp();
        for (int d = lane; d < 256; d += 32) sm.warp_hist[w][d] += sm.chain_hist[w][d];
    }
    __syncthreads();
    // per-digit counts: exclusive prefix over warps, tile total
    uint32_t count = 0;
#pragma unroll
    for (int k = 0; k < kSortWarps; ++k) {
        if (dig_thread) {
            uint32_t c = sm.warp_hist[k][tid];
            sm.warp_hist[k][tid] = count;
            count += c;
        }
    }
    uint32_t dstart = block_excl_scan256(count, sm.scan_tmp);
    if (dig_thread) {
        sm.digit_start[tid] = dstart;
        // a digit that no tile holds (its global count is 0: the last pass of
        // 30-bit keys has 64 live digits of 256) needs no look-back; no tile
        // publishes or reads its words
        const bool live = !PTGPU_SKIP_EMPTY_DIGITS || gcount != 0u;
        const uint32_t excl = live ? lookback_digit(status, tile, tid, count, st, sm.abort) : 0u;
        sm.tile_excl[tid] = goff + excl - dstart;   // + tile position = destination (mod 2^32)
    }
    __syncthreads();
    // scatter into shared memory in tile-sorted order
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        if (rank[j] != 0xffffffffu) {
            uint32_t dig = (key[j] >> shift) & 255u;
            uint32_t pos = sm.digit_start[dig] + sm.warp_hist[w][dig] + rank[j];
            sm.u.st.keys[pos] = key[j];
            const int64_t idx = base + (int64_t)w * 32 * kSortItems + j * 32 + lane;
            sm.u.st.vals[pos] = FIRST ? (int32_t)idx : ld_hint_s32<kL2Sort>(vals_in + idx);
        }
    }
    __syncthreads();
    if (sm.abort) return;
    const int valid_cnt = (int)min((int64_t)kSortTile, (int64_t)n - (int64_t)base);
    for (int i = tid; i < valid_cnt; i += kSortThreads) {
        uint32_t k = sm.u.st.keys[i];
        uint32_t dig = (k >> shift) & 255u;
        uint32_t dest = sm.tile_excl[dig] + (uint32_t)i;
        if (dest < (uint32_t)n) {
            if (!LAST) st_hint_u32<kL2Sort>(keys_out + dest, k);
            st_hint_u32<kL2Sort>(reinterpret_cast<uint32_t *>(vals_out) + dest, (uint32_t)sm.u.st.vals[i]);
        }
    }
}

// ---------------------------------------------------------------------------
// emission + refit
//
// One CTA per 1024-leaf tile.  Leaves: gather the sorted shape's vertices,
// compute its bound, stage the 60-byte leaf records in shared memory and
// copy them out as coalesced words.  Internal nodes whose range lies inside
// the tile: merge the bounds level by level in shared memory (left then
// right, as merge_bounds does), stage their records and copy out the ones the
// tile owns.  The nodes above the tiles are emitted by a climb: the tile's
// bound goes to a per-level array, and of the two tiles (then blocks) under
// a parent the one that arrives second merges them and moves up.
// ---------------------------------------------------------------------------
constexpr int kTileLog = 10;
constexpr int kTileLeaves = 1 << kTileLog;
constexpr int kTileThreads = kTileLeaves / 2;   // two leaves per thread
constexpr int kRecWords = 15;
// staged records, the 16 warps' bounds, node flags
constexpr size_t kTileSmem = kTileLeaves * kRecWords * 4 + 16 * 6 * sizeof(float) + kTileLeaves;

__device__ __forceinline__ void write_node(ptgpu_bvh_node *dst, int mn, int mx, int nshape, int leaf,
                                           int nl, int nr, int np, const float b[6], uint32_t cost_bits,
                                           uint32_t area_bits) {
    int *d = reinterpret_cast<int *>(dst);
    d[0] = mn; d[1] = mx; d[2] = nshape; d[3] = leaf; d[4] = nl; d[5] = nr; d[6] = np;
    float *f = reinterpret_cast<float *>(dst) + 7;
    for (int a = 0; a < 6; ++a) f[a] = b[a];
    d[13] = (int)cost_bits; d[14] = (int)area_bits;
}

__device__ __forceinline__ void stage_node(uint32_t *rec, int mn, int mx, int nshape, int leaf,
                                           int nl, int nr, int np, const float b[6],
                                           uint32_t cost_bits, uint32_t area_bits) {
    rec[0] = (uint32_t)mn; rec[1] = (uint32_t)mx; rec[2] = (uint32_t)nshape; rec[3] = (uint32_t)leaf;
    rec[4] = (uint32_t)nl; rec[5] = (uint32_t)nr; rec[6] = (uint32_t)np;
    for (int a = 0; a < 6; ++a) rec[7 + a] = __float_as_uint(b[a]);
    rec[13] = cost_bits; rec[14] = area_bits;
}

__device__ __forceinline__ void merge6(float *a, const float *b) {   // merge_bounds(a, b)
    a[0] = min2f(a[0], b[0]); a[1] = max2f(a[1], b[1]);
    a[2] = min2f(a[2], b[2]); a[3] = max2f(a[3], b[3]);
    a[4] = min2f(a[4], b[4]); a[5] = max2f(a[5], b[5]);
}

// The nodes above the blocks of 2^base_log leaves that one CTA emits: the
// block's bound goes to a per-level array, and of the two blocks under a
// parent the one that arrives second merges them, writes the parent's record
// and moves up.  `j` is the CTA's block, `b` its bound; per-level arrays are
// laid out level after level (nblocks, then ceil(nblocks/2), ...).
__device__ __forceinline__ void climb_blocks(int base_log, int j, float b[6], int n,
                                             ptgpu_bvh_node *__restrict__ btn,
                                             float *__restrict__ block_bounds,
                                             uint32_t *__restrict__ arrivals, int nblocks) {
    int level = base_log;
    int off = 0;                                           // first block of `level`
    for (;;) {
        float *mine = block_bounds + 6 * (size_t)(off + j);
        for (int a = 0; a < 6; ++a) mine[a] = b[a];
        if ((1 << level) >= n) break;                      // this block is the root's
        const int noff = off + ((nblocks + (1 << (level - base_log)) - 1) >> (level - base_log));
        const int pj = j >> 1;
        const int64_t right_lo = ((int64_t)(2 * pj + 1)) << level;
        if (right_lo >= n) {                               // parent has no right half
            level++; j = pj; off = noff;
            continue;
        }
        __threadfence();
        if (atomicAdd(&arrivals[noff + pj], 1u) == 0u) return;   // sibling not done yet
        __threadfence();
        const float *lbp = block_bounds + 6 * (size_t)(off + 2 * pj);
        const float *rbp = block_bounds + 6 * (size_t)(off + 2 * pj + 1);
        for (int a = 0; a < 6; ++a) b[a] = __ldcg(lbp + a);
        float c[6];
        for (int a = 0; a < 6; ++a) c[a] = __ldcg(rbp + a);
        merge6(b, c);
        level++;
        const int lo = (int)((int64_t)pj << level);
        const int64_t he = (int64_t)lo + ((int64_t)1 << level);
        const int hi = (int)((he < n ? he : n) - 1);
        const TopoBlock bn = topo_block_fast(lo, hi, level, n);
        write_node(&btn[bn.idx], lo, hi, 0, bn.leaf, bn.gamma, bn.gamma + 1, bn.parent, b, 0u, 0u);
        j = pj;
        off = noff;
    }
}

// Leaf records of every tree, and the leaves' bounds in sorted order for the
// tile kernel: one thread per leaf gathers its shape's 32-byte bound; the
// 60-byte records leave through shared memory as coalesced words.  With
// n_segs > 0 the leaves belong to the segments of seg_off (record fields are
// segment-local), otherwise to one tree of n_total leaves.
constexpr int kLeafThreads = 256;
__global__ void __launch_bounds__(kLeafThreads) k_leaves(const float4 *__restrict__ aabbs,
                                                          const int32_t *__restrict__ sorted,
                                                          int n_total, const int32_t *__restrict__ seg_off,
                                                          int n_segs, ptgpu_bvh_node *__restrict__ btl,
                                                          float4 *__restrict__ lb) {
    __shared__ uint32_t rec[kLeafThreads * kRecWords];
    __shared__ int32_t s_off[kMaxSegments + 1];
    if (n_segs > 0) {
        for (int i = threadIdx.x; i <= n_segs; i += kLeafThreads) s_off[i] = seg_off[i];
        __syncthreads();
    }
    const int k0 = blockIdx.x * kLeafThreads;
    const int k = k0 + threadIdx.x;
    if (k < n_total) {
        int off = 0, n = n_total;
        if (n_segs > 0) {
            const int g = (int)segment_of(s_off, n_segs, k);
            off = s_off[g];
            n = s_off[g + 1] - off;
        }
        // in bounds even after a failed sort
        const int sh = min(max(__ldg(sorted + k) - off, 0), n - 1) + off;
        const float4 q0 = __ldg(aabbs + 2 * (size_t)sh), q1 = __ldg(aabbs + 2 * (size_t)sh + 1);
        lb[2 * (size_t)k] = q0;
        lb[2 * (size_t)k + 1] = q1;
        const float b[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
        const int parent = n >= 2 ? topo_parent_leaf(k - off, n) : -1;
        stage_node(rec + threadIdx.x * kRecWords, -1, -1, sh - off, -1, -1, -1, parent, b, 0xffffffffu,
                   0xffffffffu);
    }
    __syncthreads();
    const int cnt = min(kLeafThreads, n_total - k0);
    uint32_t *dst = reinterpret_cast<uint32_t *>(btl + k0);
    for (int w = threadIdx.x; w < cnt * kRecWords; w += kLeafThreads) dst[w] = rec[w];
}

// One tile of one tree: `tile` counts the tree's tiles, `lb` holds the tree's
// leaf bounds in sorted order; btn/block_bounds/arrivals are the tree's own
// arrays.  The tile's internal nodes are the blocks of 2^L leaves at levels
// L = 1..10 (the index-prefix topology).  Thread t holds the leaves
// [2t, 2t+1]; levels 2-6 merge a block with its right neighbour's bound, held
// 2^(L-2) lanes up (shuffle); levels 7-10 run in warp 0 over the 16 warps'
// bounds.  A block whose right half is empty creates no node and keeps its
// bound.  Records are staged in shared memory (the active lanes of a level
// are 2^(L-1) apart, so a staging store meets at most two lanes per bank)
// and copied out as coalesced words.
template <int kSpan>
__device__ __forceinline__ void block_record(uint32_t *rec, unsigned char *own, int T0, int l0,
                                             int level, int n, const float b[6]) {
    const int lo = T0 + l0;
    const int hi = min(T0 + l0 + (1 << level), n) - 1;
    const TopoBlock bn = topo_block_fast(lo, hi, level, n);
    const int j = bn.idx - T0;
    if (bn.idx >= 0 && bn.idx < n - 1 && j >= 0 && j < kSpan) {         // internal, in the window
        stage_node(rec + j * kRecWords, lo, hi, 0, bn.leaf, bn.gamma, bn.gamma + 1, bn.parent, b, 0u, 0u);
        own[j] = 1;
    }
}

__device__ __forceinline__ void shfl_down6(float *c, const float *b, int off) {
#pragma unroll
    for (int a = 0; a < 6; ++a) c[a] = __shfl_down_sync(0xffffffffu, b[a], off);
}

__device__ __forceinline__ void emit_tile(int tile, const float4 *__restrict__ lb, int n,
                                          ptgpu_bvh_node *__restrict__ btn,
                                          float *__restrict__ block_bounds,
                                          uint32_t *__restrict__ arrivals, int ntiles,
                                          unsigned char *tsm) {
    static_assert(kTileLeaves == 1024 && kTileThreads == 512, "16 warps of 64 leaves");
    uint32_t *rec = reinterpret_cast<uint32_t *>(tsm);                      // [1024][15]
    float *wb = reinterpret_cast<float *>(rec + kTileLeaves * kRecWords);    // [16][6]
    unsigned char *own = reinterpret_cast<unsigned char *>(wb + 16 * 6);     // [1024]
    const int T0 = tile * kTileLeaves;
    const int cnt = min(kTileLeaves, n - T0);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    own[2 * tid] = 0;
    own[2 * tid + 1] = 0;
    // ---- level 1: a thread's two leaves
    const int l0 = 2 * tid;
    float b[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, c[6];
    bool have = l0 < cnt;
    if (have) {
        const float4 *p = lb + 2 * (size_t)(T0 + l0);
        const float4 q0 = __ldg(p), q1 = __ldg(p + 1);
        b[0] = q0.x; b[1] = q0.y; b[2] = q0.z; b[3] = q0.w; b[4] = q1.x; b[5] = q1.y;
        if (l0 + 1 < cnt) {
            const float4 r0 = __ldg(p + 2), r1 = __ldg(p + 3);
            c[0] = r0.x; c[1] = r0.y; c[2] = r0.z; c[3] = r0.w; c[4] = r1.x; c[5] = r1.y;
            merge6(b, c);
        }
    }
    __syncthreads();                                // own[] cleared
    if (have && l0 + 1 < cnt) block_record<kTileLeaves>(rec, own, T0, l0, 1, n, b);
    // ---- levels 2-6 inside the warp
#pragma unroll
    for (int level = 2; level <= 6; ++level) {
        const int off = 1 << (level - 2);           // lanes between a block's halves
        shfl_down6(c, b, off);
        const bool leader = (lane & ((off << 1) - 1)) == 0;
        if (leader && have && l0 + (1 << (level - 1)) < cnt) {
            merge6(b, c);
            block_record<kTileLeaves>(rec, own, T0, l0, level, n, b);
        }
    }
    if (lane == 0 && have)
        for (int a = 0; a < 6; ++a) wb[w * 6 + a] = b[a];
    __syncthreads();
    // ---- levels 7-10 over the 16 warps, in warp 0
    if (w == 0) {
        const int wl0 = 64 * lane;                  // lane j holds warp j's block
        have = lane < 16 && wl0 < cnt;
        if (have)
            for (int a = 0; a < 6; ++a) b[a] = wb[lane * 6 + a];
#pragma unroll
        for (int level = 7; level <= 10; ++level) {
            const int off = 1 << (level - 7);
            shfl_down6(c, b, off);
            const bool leader = (lane & ((off << 1) - 1)) == 0;
            if (leader && have && wl0 + (1 << (level - 1)) < cnt) {
                merge6(b, c);
                block_record<kTileLeaves>(rec, own, T0, wl0, level, n, b);
            }
        }
    }
    __syncthreads();
    {
        uint32_t *dst = reinterpret_cast<uint32_t *>(btn + T0);
        const int last = min(kTileLeaves, n - 1 - T0);     // internal indices < n-1
        for (int q = tid; q < last * kRecWords; q += kTileThreads)
            if (own[q / kRecWords]) dst[q] = rec[q];
    }
    // ---- climb above the tile (one thread, holding the tile's bound)
    if (tid != 0 || n <= kTileLeaves) return;
    climb_blocks(kTileLog, tile, b, n, btn, block_bounds, arrivals, ntiles);
}

__global__ void __launch_bounds__(kTileThreads) k_tiles(const float4 *__restrict__ lb, int n,
                                                         ptgpu_bvh_node *__restrict__ btn,
                                                         float *__restrict__ block_bounds,
                                                         uint32_t *__restrict__ arrivals, int ntiles) {
    extern __shared__ __align__(16) unsigned char tsm[];
    emit_tile(blockIdx.x, lb, n, btn, block_bounds, arrivals, ntiles, tsm);
}

// Single-tree emission (the batched build keeps k_leaves + k_tiles_seg).
// k_emit: persistent CTAs of 256 threads walk the 256-leaf windows
// [k0, k0 + 255].  Each thread gathers its sorted shape's 32-byte bound and
// stages the leaf record; the records leave as coalesced 16-byte words.  The
// bounds stay in registers for the internal nodes inside the window -- the
// blocks of 2^L leaves at L = 1..5 by warp shuffles (a block merges with its
// right half, 2^(L-1) lanes up), L = 6..8 in warp 0 over the 8 warps'
// bounds.  The level 1-5 nodes of a warp (31 of them) are then built one per
// lane from their bounds, parked in shared memory, so the topology and the
// record staging run on all lanes instead of one leader per block.  Their
// records are numbered lo or hi, so inside [k0, k0 + 255], and are copied
// out where the window owns them.  The next window's gather is issued
// before the current window is emitted, so every CTA keeps loads in flight.
// The window's bound goes to win_bounds.  k_emit_upper then does the same
// over the windows (levels 9-16, one CTA per 256 windows) and climbs above.
#ifndef PTGPU_EMIT_MINBLOCKS
#define PTGPU_EMIT_MINBLOCKS 6
#endif
constexpr int kEmitLog = 8;
constexpr int kEmitLeaves = 1 << kEmitLog;
constexpr int kUpperLog = 2 * kEmitLog;          // leaves under one k_emit_upper CTA
static_assert(kEmitLeaves == kLeafThreads, "one leaf per thread");

// PTGPU_EMIT_INDEX_AHEAD=1: each leaf's entry of `sorted` is loaded one
// window before its bound record, so the record's address is known when the
// gather is issued (otherwise the index load's latency is waited out first)
#ifndef PTGPU_EMIT_INDEX_AHEAD
#define PTGPU_EMIT_INDEX_AHEAD 1
#endif
// idx: the leaf's entry of `sorted`
__device__ __forceinline__ void gather_bound(const float4 *__restrict__ aabbs, int idx, int n,
                                             int &sh, float4 &q0, float4 &q1) {
    sh = min(max(idx, 0), n - 1);   // in bounds even after a failed sort
    q0 = ld_hint_f4<kL2Gather>(aabbs + 2 * (size_t)sh);
    q1 = ld_hint_f4<kL2Gather>(aabbs + 2 * (size_t)sh + 1);
}

// stages the record of the block at `level` starting at leaf T0 + l0 into
// its slot (index - T0) of the window, when it is an internal node there
__device__ __forceinline__ void stage_block(uint32_t *rec, int T0, int l0, int level, int n, const float b[6]) {
    const int lo = T0 + l0;
    const int hi = min(T0 + l0 + (1 << level), n) - 1;
    const TopoBlock bn = topo_block_fast(lo, hi, level, n);
    const int j = bn.idx - T0;
    if (bn.idx >= 0 && bn.idx < n - 1 && j >= 0 && j < kEmitLeaves)
        stage_node(rec + j * kRecWords, lo, hi, 0, bn.leaf, bn.gamma, bn.gamma + 1, bn.parent, b, 0u, 0u);
}

__global__ void __launch_bounds__(kLeafThreads, PTGPU_EMIT_MINBLOCKS) k_emit(const float4 *__restrict__ aabbs,
                                                        const int32_t *__restrict__ sorted, int n,
                                                        ptgpu_bvh_node *__restrict__ btl,
                                                        ptgpu_bvh_node *__restrict__ btn,
                                                        float *__restrict__ win_bounds, int nblocks) {
    pdl_begin();
#if PTGPU_PDL
    // k_emit_upper (64 CTAs for 4M leaves) may launch and wait beside this
    // persistent grid, which leaves room for it on every SM
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
    __shared__ __align__(16) uint32_t rec[kEmitLeaves * kRecWords];
    __shared__ float slot_b[8][32 * 7];     // per warp: the bounds of its 31 nodes, 7 floats apart
    __shared__ float wb[8 * 6];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    float *sb = slot_b[w];
    int win = blockIdx.x;
    int sh = 0;
    float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0;
    auto index_of = [&](int wv) {   // the entry of `sorted` for window wv's leaf tid, if any
        const int k = wv * kEmitLeaves + tid;
        return wv < nblocks && k < n ? ld_hint_s32<kL2Gather>(sorted + k) : 0;
    };
    if (win < nblocks && win * kEmitLeaves + tid < n) gather_bound(aabbs, index_of(win), n, sh, q0, q1);
    int idx_next = PTGPU_EMIT_INDEX_AHEAD ? index_of(win + (int)gridDim.x) : 0;
    for (; win < nblocks; win += gridDim.x) {
        const int k0 = win * kEmitLeaves;
        const int cnt = min(kEmitLeaves, n - k0);
        const bool have = tid < cnt;
        const int kn = (win + (int)gridDim.x) * kEmitLeaves + tid;
        const bool have_n = win + (int)gridDim.x < nblocks && kn < n;
        float b[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y}, c[6];
        if (have) {
            const int parent = n >= 2 ? topo_parent_leaf_fast(k0 + tid, n) : -1;
            stage_node(rec + tid * kRecWords, -1, -1, sh, -1, -1, -1, parent, b, 0xffffffffu, 0xffffffffu);
        }
        // ---- levels 1-5 inside the warp; level L parks its bounds in
        // slots 32 - 2^(6-L) ...
#pragma unroll
        for (int level = 1; level <= 5; ++level) {
            const int off = 1 << (level - 1);
            shfl_down6(c, b, off);
            const bool leader = (lane & ((off << 1) - 1)) == 0;
            if (leader && have && tid + off < cnt) {
                merge6(b, c);
                const int slot = 32 - (64 >> level) + (lane >> level);
#pragma unroll
                for (int a = 0; a < 6; ++a) sb[slot * 7 + a] = b[a];
            }
        }
        if (lane == 0 && have)
            for (int a = 0; a < 6; ++a) wb[w * 6 + a] = b[a];
        __syncthreads();
        // ---- the next window's gather, in flight while this one is emitted
        if (PTGPU_EMIT_INDEX_AHEAD) {
            if (have_n) gather_bound(aabbs, idx_next, n, sh, q0, q1);
            idx_next = index_of(win + 2 * (int)gridDim.x);
        } else if (have_n) {
            gather_bound(aabbs, index_of(win + (int)gridDim.x), n, sh, q0, q1);
        }
        {   // the window's records start on a 16-byte boundary (256 * 60 bytes per window)
            uint32_t *dst = reinterpret_cast<uint32_t *>(btl + k0);
            const int words = cnt * kRecWords, chunks = words >> 2;
            for (int q = tid; q < chunks; q += kLeafThreads)
                st_hint_u4<kL2Nodes>(reinterpret_cast<uint4 *>(dst) + q, reinterpret_cast<const uint4 *>(rec)[q]);
            for (int q = 4 * chunks + tid; q < words; q += kLeafThreads) st_hint_u32<kL2Nodes>(dst + q, rec[q]);
        }
        __syncthreads();                            // staging buffer free
        // ---- the warp's level 1-5 nodes, one per lane (lane 31 idle)
        if (lane < 31) {
            const int level = 6 - (32 - __clz(31 - lane));           // 6 - ceil(log2(32 - lane))
            const int lo_w = (lane - (32 - (64 >> level))) << level;  // first leaf in the warp
            if (32 * w + lo_w + (1 << (level - 1)) < cnt) {          // right half non-empty
                float nb[6];
#pragma unroll
                for (int a = 0; a < 6; ++a) nb[a] = sb[lane * 7 + a];
                stage_block(rec, k0, 32 * w + lo_w, level, n, nb);
            }
        }
        // ---- levels 6-8 over the 8 warps, in warp 0
        if (w == 0) {
            const int wl0 = 32 * lane;              // lane j holds warp j's block
            const bool h = lane < 8 && wl0 < cnt;
            if (h)
                for (int a = 0; a < 6; ++a) b[a] = wb[lane * 6 + a];
#pragma unroll
            for (int level = 6; level <= 8; ++level) {
                const int off = 1 << (level - 6);
                shfl_down6(c, b, off);
                const bool leader = (lane & ((off << 1) - 1)) == 0;
                if (leader && h && wl0 + (1 << (level - 1)) < cnt) {
                    merge6(b, c);
                    stage_block(rec, k0, wl0, level, n, b);
                }
            }
            if (lane == 0)
                for (int a = 0; a < 6; ++a) win_bounds[6 * (size_t)win + a] = b[a];
        }
        __syncthreads();
        {   // every slot of the window: the one slot (at most) that belongs to a
            // node above the window gets a stale record here, which
            // k_emit_upper overwrites after this kernel ends
            uint32_t *dst = reinterpret_cast<uint32_t *>(btn + k0);
            const int last = min(kEmitLeaves, n - 1 - k0);     // internal indices < n-1
            const int words = max(last, 0) * kRecWords, chunks = words >> 2;
            for (int q = tid; q < chunks; q += kLeafThreads)
                st_hint_u4<kL2Nodes>(reinterpret_cast<uint4 *>(dst) + q, reinterpret_cast<const uint4 *>(rec)[q]);
            for (int q = 4 * chunks + tid; q < words; q += kLeafThreads) st_hint_u32<kL2Nodes>(dst + q, rec[q]);
        }
        __syncthreads();                            // rec and the slots are reused
    }
}

// record of the block at `level` starting at leaf lo, written in place
__device__ __forceinline__ void upper_record(int lo, int level, int n, const float b[6],
                                             ptgpu_bvh_node *__restrict__ btn) {
    const int hi = (int)min((int64_t)lo + ((int64_t)1 << level), (int64_t)n) - 1;
    const TopoBlock bn = topo_block_fast(lo, hi, level, n);
    if (bn.idx >= 0 && bn.idx < n - 1)
        write_node(&btn[bn.idx], lo, hi, 0, bn.leaf, bn.gamma, bn.gamma + 1, bn.parent, b, 0u, 0u);
}

// Levels base+1 .. base+8 over 256 units of 2^base leaves each (unit u0 +
// thread), their bounds in b: levels base+1..base+5 by warp shuffles, the
// rest in warp 0 over the 8 warps' bounds; records written in place.  On
// return thread 0 holds the bound of all 256 units.
__device__ __forceinline__ void reduce_units(float b[6], int u0, int nunits, int base, int n,
                                             ptgpu_bvh_node *__restrict__ btn, float *wb) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int u = u0 + tid;
    const bool have = u < nunits;
    float c[6];
#pragma unroll
    for (int m = 1; m <= 5; ++m) {
        const int off = 1 << (m - 1);
        shfl_down6(c, b, off);
        const bool leader = (lane & ((off << 1) - 1)) == 0;
        if (leader && have && u + off < nunits) {
            merge6(b, c);
            upper_record(u << base, base + m, n, b, btn);
        }
    }
    if (lane == 0 && have)
        for (int a = 0; a < 6; ++a) wb[w * 6 + a] = b[a];
    __syncthreads();
    if (w == 0) {
        const int ul = u0 + 32 * lane;              // lane j holds warp j's 32 units
        const bool h = lane < 8 && ul < nunits;
        if (h)
            for (int a = 0; a < 6; ++a) b[a] = wb[lane * 6 + a];
#pragma unroll
        for (int m = 6; m <= 8; ++m) {
            const int off = 1 << (m - 6);
            shfl_down6(c, b, off);
            const bool leader = (lane & ((off << 1) - 1)) == 0;
            if (leader && h && ul + (1 << (m - 1)) < nunits) {
                merge6(b, c);
                upper_record(ul << base, base + m, n, b, btn);
            }
        }
    }
}

// The nodes above the windows: one CTA per 256 windows (2^16 leaves) builds
// levels 9-16 from the window bounds.  Up to 256 such CTAs (2^24 leaves),
// the CTA that finishes last builds levels 17-24 from their bounds the same
// way; above that each CTA climbs with arrival counters.
__global__ void __launch_bounds__(256) k_emit_upper(const float *__restrict__ win_bounds, int nblocks, int n,
                                                    ptgpu_bvh_node *__restrict__ btn,
                                                    float *__restrict__ super_bounds,
                                                    uint32_t *__restrict__ arrivals, int nsuper) {
    pdl_begin();
    __shared__ float wb[8 * 6];
    __shared__ int s_last;
    const int tid = threadIdx.x;
    const int u0 = blockIdx.x * 256;
    float b[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (u0 + tid < nblocks)
        for (int a = 0; a < 6; ++a) b[a] = win_bounds[6 * (size_t)(u0 + tid) + a];
    reduce_units(b, u0, nblocks, kEmitLog, n, btn, wb);
    if (n <= (1 << kUpperLog)) return;              // the root was built above
    if (nsuper > 256) {
        if (tid == 0) climb_blocks(kUpperLog, blockIdx.x, b, n, btn, super_bounds, arrivals, nsuper);
        return;
    }
    if (tid == 0) {
        for (int a = 0; a < 6; ++a) super_bounds[6 * (size_t)blockIdx.x + a] = b[a];
        __threadfence();
        s_last = atomicAdd(&arrivals[0], 1u) == (uint32_t)(nsuper - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    if (tid < nsuper)
        for (int a = 0; a < 6; ++a) b[a] = __ldcg(super_bounds + 6 * (size_t)tid + a);
    __syncthreads();                                // wb reused
    reduce_units(b, 0, nsuper, kUpperLog, n, btn, wb);
}

// the tiles of every segment's tree in one launch
__global__ void __launch_bounds__(kTileThreads) k_tiles_seg(const float4 *__restrict__ lb, SegBuild sb,
                                                             ptgpu_bvh_node *__restrict__ btn,
                                                             float *__restrict__ block_bounds,
                                                             uint32_t *__restrict__ arrivals) {
    extern __shared__ __align__(16) unsigned char tsm[];
    const int t = blockIdx.x;
    const int g = (int)segment_of(sb.tile_off, sb.n_segs, t);
    const int off = sb.seg_off[g], n = sb.seg_off[g + 1] - off;
    const int tile = t - sb.tile_off[g];
    const int64_t bb = sb.bb_off[g];
    emit_tile(tile, lb + 2 * (size_t)off, n, btn + (off - g), block_bounds + 6 * bb, arrivals + bb,
              sb.tile_off[g + 1] - sb.tile_off[g], tsm);
}

// ---------------------------------------------------------------------------
// Treelet restructuring (Karras & Aila, "Fast Parallel Construction of
// High-Quality Bounding Volume Hierarchies", HPG 2013), the stage that
// kernelOptimize / treeletOptimize (BVH.cl:291-543) set out to implement:
// bottom-up over the tree with atomic arrival counters; at each node the
// treelet of up to 7 leaves is grown by expanding the largest-area child,
// the optimal binary topology over those leaves is found by dynamic
// programming over all 127 subsets with SAH cost Ci*A + children (Ci = 1.2,
// leaf cost Ct*A with Ct = 1.0, clheader.h:14-15), and the treelet is rebuilt
// in place when that is strictly cheaper.  Internal nodes mark a leaf child
// with min == nLeft / max == nRight and an internal child with -1.  One
// thread per treelet; the float operations and their order are those of the
// oracle's sequential restatement, so the two trees agree byte for byte.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float area6(const float *b) {
    float dx = b[1] - b[0], dy = b[3] - b[2], dz = b[5] - b[4];
    return 2.f * (dx * dy + dx * dz + dy * dz);
}

// Nodes and costs written by other threads are read past L1 (ld.global.cg):
// a node's subtree was finished on another SM before its arrival counter
// let this thread in.
struct NodeL {
    int min, max, leaf, nLeft, nRight, nParent;
};
__device__ __forceinline__ NodeL load_node(const ptgpu_bvh_node *btn, int i) {
    const int *w = reinterpret_cast<const int *>(btn + i);
    NodeL n;
    n.min = __ldcg(w + 0); n.max = __ldcg(w + 1); n.leaf = __ldcg(w + 3);
    n.nLeft = __ldcg(w + 4); n.nRight = __ldcg(w + 5); n.nParent = __ldcg(w + 6);
    return n;
}
__device__ __forceinline__ void ref_bound6(int r, const ptgpu_bvh_node *btn,
                                           const ptgpu_bvh_node *btl, float *b) {
    const float *x = reinterpret_cast<const float *>(r < 0 ? btl + (-r - 1) : btn + r) + 7;
    for (int a = 0; a < 6; ++a) b[a] = __ldcg(x + a);
}

__device__ __forceinline__ int child_ref(const NodeL &nd, bool right) {
    if (!right) return nd.nLeft == nd.min ? -(nd.nLeft + 1) : nd.nLeft;
    return nd.nRight == nd.max ? -(nd.nRight + 1) : nd.nRight;
}

__device__ __forceinline__ float ref_cost(int r, const float *cost, const ptgpu_bvh_node *btl) {
    if (r >= 0) return __ldcg(cost + r);
    float b[6];
    ref_bound6(r, nullptr, btl, b);
    return 1.0f * area6(b);
}

// normalise child marks: min = nLeft for a leaf left child else -1, likewise max
__global__ void k_treelet_prepare(ptgpu_bvh_node *btn, int n, int *counters) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    ptgpu_bvh_node &p = btn[i];
    bool ll = p.nLeft == p.min, rl = p.nRight == p.max;
    p.min = ll ? p.nLeft : -1;
    p.max = rl ? p.nRight : -1;
    counters[i] = 0;
}

// Subsets of 7 leaves ordered by (size, value); kSubsetStart[k] is where the
// subsets of size k begin.  Within a size the first C(nl, k) entries are the
// subsets of the first nl leaves.
__device__ const unsigned char kSubsets[127] = {
    1, 2, 4, 8, 16, 32, 64,
    3, 5, 6, 9, 10, 12, 17, 18, 20, 24, 33, 34, 36, 40, 48, 65, 66, 68, 72, 80, 96,
    7, 11, 13, 14, 19, 21, 22, 25, 26, 28, 35, 37, 38, 41, 42, 44, 49, 50, 52, 56, 67, 69, 70,
    73, 74, 76, 81, 82, 84, 88, 97, 98, 100, 104, 112,
    15, 23, 27, 29, 30, 39, 43, 45, 46, 51, 53, 54, 57, 58, 60, 71, 75, 77, 78, 83, 85, 86, 89,
    90, 92, 99, 101, 102, 105, 106, 108, 113, 114, 116, 120,
    31, 47, 55, 59, 61, 62, 79, 87, 91, 93, 94, 103, 107, 109, 110, 115, 117, 118, 121, 122, 124,
    63, 95, 111, 119, 123, 125, 126,
    127};
__device__ const unsigned char kSubsetStart[8] = {0, 0, 7, 28, 63, 98, 119, 126};

__device__ const unsigned char kBinom7[8][8] = {   // C(n, k), n, k <= 7
    {1, 0, 0, 0, 0, 0, 0, 0},     {1, 1, 0, 0, 0, 0, 0, 0},     {1, 2, 1, 0, 0, 0, 0, 0},
    {1, 3, 3, 1, 0, 0, 0, 0},     {1, 4, 6, 4, 1, 0, 0, 0},     {1, 5, 10, 10, 5, 1, 0, 0},
    {1, 6, 15, 20, 15, 6, 1, 0},  {1, 7, 21, 35, 35, 21, 7, 1}};
// the (x)-th subset of `mask`: the low bits of x deposited on mask's set bits
__device__ __forceinline__ int deposit(int x, int mask) {
    int r = 0;
    for (int m = mask; m; m &= m - 1) {
        if (x & 1) r |= m & -m;
        x >>= 1;
    }
    return r;
}

// Per-warp scratch of one treelet.
struct TreeletSmem {
    float lb[7][6];     // bounds of the treelet's leaves
    float la[7];        // their areas (expansion candidates)
    float area[128];
    float copt[128];
    unsigned char popt[128];
    int leaves[7];
    int nodes[6];
};

// One treelet, all 32 lanes of the warp.  Formation, subset areas and the
// dynamic programme run across the lanes; every float result is produced by
// the same operations in the same order as the sequential restatement:
// unions merge a subset's leaves in index order, and the best split of a
// subset is the first partition, in the enumeration p = (p - d) & s, with the
// least cost (each lane scans its share of the partitions in that order, and
// ties between lanes go to the earlier partition).  Bounds and costs read
// once from memory are kept in shared memory and reused where the
// sequential code reads them again.
__device__ void treelet_warp(int root, float root_cost, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl,
                             float *cost, TreeletSmem &sm, int lane) {
    if (lane == 0) {
        const NodeL r = load_node(btn, root);
        sm.leaves[0] = child_ref(r, false);
        sm.leaves[1] = child_ref(r, true);
    }
    __syncwarp();
    if (lane < 2) {
        ref_bound6(sm.leaves[lane], btn, btl, sm.lb[lane]);
        sm.la[lane] = area6(sm.lb[lane]);
    }
    __syncwarp();
    int nl = 2, nn = 0;
    while (nl < 7) {
        // expand the internal leaf of largest area (first index on ties)
        float a = -1.f;
        int bi = 32;
        if (lane < nl && sm.leaves[lane] >= 0 && sm.la[lane] > -1.f) { a = sm.la[lane]; bi = lane; }
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const float oa = __shfl_xor_sync(0xffffffffu, a, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (oi < 32 && (bi == 32 || oa > a || (oa == a && oi < bi))) { a = oa; bi = oi; }
        }
        bi = __shfl_sync(0xffffffffu, bi, 0);
        if (bi == 32) break;
        if (lane == 0) {
            const int nd = sm.leaves[bi];
            sm.nodes[nn] = nd;
            const NodeL x = load_node(btn, nd);
            sm.leaves[bi] = child_ref(x, false);
            sm.leaves[nl] = child_ref(x, true);
        }
        __syncwarp();
        if (lane < 2) {
            const int slot = lane == 0 ? bi : nl;
            ref_bound6(sm.leaves[slot], btn, btl, sm.lb[slot]);
            sm.la[slot] = area6(sm.lb[slot]);
        }
        __syncwarp();
        ++nn;
        ++nl;
    }
    if (nl < 3) return;
    const int nsub = 1 << nl;
    if (lane < nl) {
        // ref_cost: the subtree cost of an internal node, Ct * area of a leaf
        const int r = sm.leaves[lane];
        sm.copt[1 << lane] = r >= 0 ? __ldcg(cost + r) : 1.0f * area6(sm.lb[lane]);
    }
    for (int s = lane + 1; s < nsub; s += 32) {
        float b[6];
        bool first = true;
        for (int i = 0; i < nl; i++) {
            if (!((s >> i) & 1)) continue;
            if (first) { for (int q = 0; q < 6; ++q) b[q] = sm.lb[i][q]; first = false; }
            else merge6(b, sm.lb[i]);
        }
        sm.area[s] = area6(b);
    }
    __syncwarp();
    for (int k = 2; k <= nl; k++) {
        const int cnt = kBinom7[nl][k];
        const int nparts = (1 << (k - 1)) - 1;
        int g = 1;   // lanes per subset
        while (g < nparts && 2 * g * cnt <= 32) g *= 2;
        for (int base = 0; base < cnt * g; base += 32) {
            const int item = base + lane;
            const bool valid = item < cnt * g;
            const int m = item / g, jj = item % g;
            const int s = valid ? kSubsets[kSubsetStart[k] + m] : 0;
            const int d = (s - 1) & s;
            float bc = FLT_MAX;
            int bj = -1;
            if (valid && g == 1) {
                int j = 0;
                for (int p = (-d) & s; p != 0; p = (p - d) & s, ++j) {
                    const float c = sm.copt[p] + sm.copt[s ^ p];
                    if (c < bc) { bc = c; bj = j; }
                }
            } else if (valid) {
                for (int j = jj; j < nparts; j += g) {
                    const int p = deposit(j + 1, d);
                    const float c = sm.copt[p] + sm.copt[s ^ p];
                    if (c < bc) { bc = c; bj = j; }
                }
            }
            for (int o = 1; o < g; o <<= 1) {
                const float oc = __shfl_xor_sync(0xffffffffu, bc, o);
                const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
                if (oj >= 0 && (bj < 0 || oc < bc || (oc == bc && oj < bj))) { bc = oc; bj = oj; }
            }
            if (valid && jj == 0) {
                sm.copt[s] = 1.2f * sm.area[s] + bc;
                sm.popt[s] = (unsigned char)(bj >= 0 ? deposit(bj + 1, d) : 0);
            }
        }
        __syncwarp();
    }
    const int full = nsub - 1;
    if (!(sm.copt[full] < root_cost)) return;
    if (lane != 0) return;
    // rebuild (one lane): internal slots are root + nodes[], reused in DFS
    // order; a child is a treelet leaf -(i+1) or a slot index
    int slot_node[7], kid[7][2];
    int ns = 0;
    slot_node[ns++] = root;
    for (int i = 0; i < nn; i++) slot_node[ns++] = sm.nodes[i];
    int used = 1;
    int st_s[8], st_u[8], top = 0;
    st_s[top] = full; st_u[top] = 0; top++;
    while (top) {
        top--;
        const int s = st_s[top], u = st_u[top], nd = slot_node[u];
        const int ls = sm.popt[s];
        const int subs[2] = {ls, s ^ ls};
        int refs[2];
        for (int c = 0; c < 2; c++) {
            if (__popc(subs[c]) == 1) {
                const int i = __ffs(subs[c]) - 1;
                kid[u][c] = -(i + 1);
                refs[c] = sm.leaves[i];
            } else {
                const int v = used++;
                kid[u][c] = v;
                refs[c] = slot_node[v];
                st_s[top] = subs[c]; st_u[top] = v; top++;
            }
        }
        ptgpu_bvh_node &p = btn[nd];
        p.nLeft = refs[0] < 0 ? -refs[0] - 1 : refs[0];
        p.nRight = refs[1] < 0 ? -refs[1] - 1 : refs[1];
        p.min = refs[0] < 0 ? p.nLeft : -1;
        p.max = refs[1] < 0 ? p.nRight : -1;
        p.leaf = (refs[0] < 0 || refs[1] < 0) ? 2 : 0;
        if (refs[0] < 0) btl[-refs[0] - 1].nParent = nd; else btn[refs[0]].nParent = nd;
        if (refs[1] < 0) btl[-refs[1] - 1].nParent = nd; else btn[refs[1]].nParent = nd;
    }
    // bounds and costs bottom-up (children have higher slot indices):
    // union of left then right, cost Ci * area + left cost + right cost
    float sb[7][6], sc[7];
    for (int u = used - 1; u >= 0; u--) {
        float b[6], cl, cr;
        const int l = kid[u][0], r = kid[u][1];
        const float *lbp = l < 0 ? sm.lb[-l - 1] : sb[l];
        const float *rbp = r < 0 ? sm.lb[-r - 1] : sb[r];
        cl = l < 0 ? sm.copt[1 << (-l - 1)] : sc[l];
        cr = r < 0 ? sm.copt[1 << (-r - 1)] : sc[r];
        for (int q = 0; q < 6; ++q) b[q] = lbp[q];
        merge6(b, rbp);
        for (int q = 0; q < 6; ++q) sb[u][q] = b[q];
        sc[u] = 1.2f * area6(b) + cl + cr;
        ptgpu_bvh_node &p = btn[slot_node[u]];
        p.bound.min_x = b[0]; p.bound.max_x = b[1]; p.bound.min_y = b[2];
        p.bound.max_y = b[3]; p.bound.min_z = b[4]; p.bound.max_z = b[5];
        cost[slot_node[u]] = sc[u];
    }
    __threadfence();
}

// Bottom-up over the tree: each lane climbs from its leaf and the second
// arrival at a node owns it.  The lanes of a warp that own a node in the same
// round hand their treelets to the whole warp one after another.
constexpr int kTreeletThreads = 128;
// Leaves a warp climbs from (its other lanes only help in the treelets):
// fewer leaves per warp put more warps, and so more treelets, in flight,
// which pays on small trees (82k-shape scene, LBVH + 2 rounds: 32 -> 1.29 ms,
// 16 -> 1.22 ms) and costs on large ones, where 32 already fill the GPU
// (17.3M leaves of a batch: build 97 ms with 16 against 81 ms with 32).
__device__ __forceinline__ int treelet_leaf(int lane, int lpw) {
    return lane < lpw ? (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * lpw + lane : 0x7fffffff;
}
#ifndef PTGPU_TREELET_LPW
#define PTGPU_TREELET_LPW 0    // leaves a warp climbs from; 0: 16 below 2^20 leaves, else 32
#endif
static int treelet_lpw(int64_t leaves) {
    return PTGPU_TREELET_LPW > 0 ? PTGPU_TREELET_LPW : (leaves < (1 << 20) ? 16 : 32);
}
static int treelet_grid(int64_t leaves, int lpw) {
    return (int)((leaves + (int64_t)lpw * (kTreeletThreads / 32) - 1) / ((int64_t)lpw * (kTreeletThreads / 32)));
}

__global__ void __launch_bounds__(kTreeletThreads) k_treelet(ptgpu_bvh_node *btn,
                                                              ptgpu_bvh_node *btl, int n,
                                                              int *counters, float *cost, int lpw) {
    __shared__ TreeletSmem s_tl[kTreeletThreads / 32];
    TreeletSmem &sm = s_tl[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int k = treelet_leaf(lane, lpw);
    int node = k < n ? btl[k].nParent : -1;
    bool active = node >= 0 && node < n - 1;
    while (__any_sync(0xffffffffu, active)) {
        bool mine = false;
        float my_cost = 0.f;
        if (active) {
            __threadfence();
            if (atomicAdd(&counters[node], 1) == 0) {
                active = false;                    // the second arrival goes on
            } else {
                __threadfence();
                // all of node's subtree is final: its cost first
                const NodeL p = load_node(btn, node);
                int lr = p.min == p.nLeft ? -(p.nLeft + 1) : p.nLeft;
                int rr = p.max == p.nRight ? -(p.nRight + 1) : p.nRight;
                float b[6];
                ref_bound6(node, btn, btl, b);
                my_cost = 1.2f * area6(b) + ref_cost(lr, cost, btl) + ref_cost(rr, cost, btl);
                cost[node] = my_cost;
                mine = true;
            }
        }
        unsigned m = __ballot_sync(0xffffffffu, mine);
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const int root = __shfl_sync(0xffffffffu, node, src);
            const float rc = __shfl_sync(0xffffffffu, my_cost, src);
            treelet_warp(root, rc, btn, btl, cost, sm, lane);
            __syncwarp();
        }
        if (mine) {
            __threadfence();
            if (node == 0) active = false;
            else node = load_node(btn, node).nParent;
            if (node < 0 || node >= n - 1) active = false;
        }
    }
}

__global__ void k_treelet_finish(ptgpu_bvh_node *btn, int n, const float *cost) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    ptgpu_bvh_node &p = btn[i];
    float b[6] = {p.bound.min_x, p.bound.max_x, p.bound.min_y, p.bound.max_y, p.bound.min_z,
                  p.bound.max_z};
    p.cost = cost[i];
    p.area = area6(b);
}

// The treelet rounds of every segment's tree in one launch per round (the
// batched build): segment g's tree has n_g = seg_off[g+1] - seg_off[g]
// leaves, its leaves at btl + seg_off[g] and its internal nodes, counters and
// costs at seg_off[g] - g, all indices inside segment-local.  Segments with
// fewer than 3 leaves are left alone, as launch_treelet leaves such a tree.
__device__ __forceinline__ int internal_segment(const int32_t *seg_off, int n_segs, int i) {
    int lo = 0, hi = n_segs - 1;          // the last g with seg_off[g] - g <= i
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (seg_off[mid] - mid <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void k_treelet_prepare_seg(ptgpu_bvh_node *btn, const int32_t *__restrict__ seg_off, int n_segs,
                                      int n_internal, int *counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_internal) return;
    const int g = internal_segment(seg_off, n_segs, i);
    if (seg_off[g + 1] - seg_off[g] < 3) return;
    ptgpu_bvh_node &p = btn[i];
    const bool ll = p.nLeft == p.min, rl = p.nRight == p.max;
    p.min = ll ? p.nLeft : -1;
    p.max = rl ? p.nRight : -1;
    counters[i] = 0;
}

__global__ void k_treelet_finish_seg(ptgpu_bvh_node *btn, const int32_t *__restrict__ seg_off, int n_segs,
                                     int n_internal, const float *cost) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_internal) return;
    const int g = internal_segment(seg_off, n_segs, i);
    if (seg_off[g + 1] - seg_off[g] < 3) return;
    ptgpu_bvh_node &p = btn[i];
    float b[6] = {p.bound.min_x, p.bound.max_x, p.bound.min_y, p.bound.max_y, p.bound.min_z,
                  p.bound.max_z};
    p.cost = cost[i];
    p.area = area6(b);
}

__global__ void __launch_bounds__(kTreeletThreads) k_treelet_seg(ptgpu_bvh_node *btn, ptgpu_bvh_node *btl,
                                                                  const int32_t *__restrict__ seg_off, int n_segs,
                                                                  int n_total, int *counters, float *cost,
                                                                  int lpw) {
    __shared__ TreeletSmem s_tl[kTreeletThreads / 32];
    TreeletSmem &sm = s_tl[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int k = treelet_leaf(lane, lpw);
    int g = 0, off = 0, n = 0;
    if (k < n_total) {
        g = (int)segment_of(seg_off, n_segs, k);
        off = seg_off[g];
        n = seg_off[g + 1] - off;
    }
    // this lane's tree: internal nodes, counters and costs at off - g
    ptgpu_bvh_node *tn = btn + (off - g), *tl = btl + off;
    int *tc = counters + (off - g);
    float *tcost = cost + (off - g);
    int node = (k < n_total && n >= 3) ? tl[k - off].nParent : -1;
    bool active = node >= 0 && node < n - 1;
    while (__any_sync(0xffffffffu, active)) {
        bool mine = false;
        float my_cost = 0.f;
        if (active) {
            __threadfence();
            if (atomicAdd(&tc[node], 1) == 0) {
                active = false;                    // the second arrival goes on
            } else {
                __threadfence();
                const NodeL p = load_node(tn, node);
                int lr = p.min == p.nLeft ? -(p.nLeft + 1) : p.nLeft;
                int rr = p.max == p.nRight ? -(p.nRight + 1) : p.nRight;
                float b[6];
                ref_bound6(node, tn, tl, b);
                my_cost = 1.2f * area6(b) + ref_cost(lr, tcost, tl) + ref_cost(rr, tcost, tl);
                tcost[node] = my_cost;
                mine = true;
            }
        }
        unsigned m = __ballot_sync(0xffffffffu, mine);
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const int root = __shfl_sync(0xffffffffu, node, src);
            const float rc = __shfl_sync(0xffffffffu, my_cost, src);
            const int sg = __shfl_sync(0xffffffffu, g, src);
            const int so = __shfl_sync(0xffffffffu, off, src);
            treelet_warp(root, rc, btn + (so - sg), btl + so, cost + (so - sg), sm, lane);
            __syncwarp();
        }
        if (mine) {
            __threadfence();
            if (node == 0) active = false;
            else node = load_node(tn, node).nParent;
            if (node < 0 || node >= n - 1) active = false;
        }
    }
}

cudaError_t launch_treelet_seg(ptgpu_bvh_node *btn, ptgpu_bvh_node *btl, const int32_t *seg_off, int n_segs,
                               int n_total, int *counters, float *cost, int sweeps, cudaStream_t s) {
    const int n_internal = n_total - n_segs;
    if (n_internal <= 0) return cudaSuccess;
    k_treelet_prepare_seg<<<(n_internal + 255) / 256, 256, 0, s>>>(btn, seg_off, n_segs, n_internal, counters);
    for (int it = 0; it < sweeps; ++it) {
        if (it > 0) cudaMemsetAsync(counters, 0, sizeof(int) * (size_t)n_internal, s);
        k_treelet_seg<<<treelet_grid(n_total, treelet_lpw(n_total)), kTreeletThreads, 0, s>>>(
            btn, btl, seg_off, n_segs, n_total, counters, cost, treelet_lpw(n_total));
    }
    k_treelet_finish_seg<<<(n_internal + 255) / 256, 256, 0, s>>>(btn, seg_off, n_segs, n_internal, cost);
    return cudaGetLastError();
}

cudaError_t launch_treelet(ptgpu_bvh_node *btn, ptgpu_bvh_node *btl, int n, int *counters,
                           float *cost, int sweeps, cudaStream_t s) {
    if (n < 3) return cudaSuccess;
    k_treelet_prepare<<<(n + 255) / 256, 256, 0, s>>>(btn, n, counters);
    for (int it = 0; it < sweeps; ++it) {
        if (it > 0) cudaMemsetAsync(counters, 0, sizeof(int) * (size_t)(n - 1), s);
        k_treelet<<<treelet_grid(n, treelet_lpw(n)), kTreeletThreads, 0, s>>>(
            btn, btl, n, counters, cost, treelet_lpw(n));
    }
    k_treelet_finish<<<(n + 255) / 256, 256, 0, s>>>(btn, n, cost);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// ABI arrays -> traversal layout (works for any btn/btl, including trees
// installed by the caller or restructured by the treelet pass): a child is a
// leaf when nLeft == min / nRight == max.
// ---------------------------------------------------------------------------
__global__ void k_abi_to_trace(const ptgpu_bvh_node *__restrict__ btn,
                               const ptgpu_bvh_node *__restrict__ btl, int n,
                               const float4 *__restrict__ prims0, float4 *__restrict__ nodes,
                               float4 *__restrict__ prims, int32_t *__restrict__ prim_id,
                               int node_base, int shape_base) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        int s = min(max(btl[i].nShape, 0), n - 1);
        prim_id[i] = shape_base + s;
        prims[3 * (size_t)i + 0] = prims0[3 * (size_t)s + 0];
        prims[3 * (size_t)i + 1] = prims0[3 * (size_t)s + 1];
        prims[3 * (size_t)i + 2] = prims0[3 * (size_t)s + 2];
    }
    if (i < n - 1) {
        const ptgpu_bvh_node nd = btn[i];
        bool ll = nd.nLeft == nd.min, rl = nd.nRight == nd.max;
        const int li = min(max(nd.nLeft, 0), ll ? n - 1 : n - 2);
        const int ri = min(max(nd.nRight, 0), rl ? n - 1 : n - 2);
        const ptgpu_bound lb = ll ? btl[li].bound : btn[li].bound;
        const ptgpu_bound rb = rl ? btl[ri].bound : btn[ri].bound;
        float4 *o = nodes + 4 * (size_t)i;
        o[0] = make_float4(lb.min_x, lb.max_x, lb.min_y, lb.max_y);
        o[1] = make_float4(lb.min_z, lb.max_z, rb.min_x, rb.max_x);
        o[2] = make_float4(rb.min_y, rb.max_y, rb.min_z, rb.max_z);
        int4 q = make_int4((ll ? shape_base : node_base) + li, (rl ? shape_base : node_base) + ri,
                           ll ? 1 : 0, rl ? 1 : 0);
        o[3] = *reinterpret_cast<float4 *>(&q);
    }
}

// Binary traversal nodes -> 4-wide nodes (see types.h): slot k holds a child
// of binary node i, an internal child being replaced by its two children.
__global__ void k_collapse4(const float4 *__restrict__ nodes2, int n_int,
                            float4 *__restrict__ nodes4) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_int) return;
    float box[4][6];
    int ref[4], cnt[4];
    int ns = 0;
    const float4 *nd = nodes2 + 4 * (size_t)i;
    float4 q0 = nd[0], q1 = nd[1], q2 = nd[2], q3 = nd[3];
    const int lref = __float_as_int(q3.x), rref = __float_as_int(q3.y);
    const int lcnt = __float_as_int(q3.z), rcnt = __float_as_int(q3.w);
    float lb[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
    float rb[6] = {q1.z, q1.w, q2.x, q2.y, q2.z, q2.w};
    for (int side = 0; side < 2; ++side) {
        const int r = side ? rref : lref, c = side ? rcnt : lcnt;
        const float *b = side ? rb : lb;
        if (c > 0 || r < 0 || r >= n_int) {
            for (int a = 0; a < 6; ++a) box[ns][a] = b[a];
            ref[ns] = r; cnt[ns] = c > 0 ? c : -1; ++ns;
            continue;
        }
        const float4 *cn = nodes2 + 4 * (size_t)r;
        float4 c0 = cn[0], c1 = cn[1], c2 = cn[2], c3 = cn[3];
        float cl[6] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y};
        float cr[6] = {c1.z, c1.w, c2.x, c2.y, c2.z, c2.w};
        for (int a = 0; a < 6; ++a) box[ns][a] = cl[a];
        ref[ns] = __float_as_int(c3.x); cnt[ns] = __float_as_int(c3.z); ++ns;
        for (int a = 0; a < 6; ++a) box[ns][a] = cr[a];
        ref[ns] = __float_as_int(c3.y); cnt[ns] = __float_as_int(c3.w); ++ns;
    }
    for (; ns < 4; ++ns) {
        box[ns][0] = box[ns][2] = box[ns][4] = 1.f;
        box[ns][1] = box[ns][3] = box[ns][5] = 0.f;
        ref[ns] = 0; cnt[ns] = -1;
    }
    float4 *o = nodes4 + 8 * (size_t)i;
    for (int a = 0; a < 6; ++a) o[a] = make_float4(box[0][a], box[1][a], box[2][a], box[3][a]);
    o[6] = make_float4(__int_as_float(ref[0]), __int_as_float(ref[1]), __int_as_float(ref[2]),
                       __int_as_float(ref[3]));
    o[7] = make_float4(__int_as_float(cnt[0]), __int_as_float(cnt[1]), __int_as_float(cnt[2]),
                       __int_as_float(cnt[3]));
}

cudaError_t launch_collapse4(const float4 *nodes2, int n_int, float4 *nodes4, cudaStream_t s) {
    if (n_int <= 0) return cudaSuccess;
    k_collapse4<<<(n_int + 255) / 256, 256, 0, s>>>(nodes2, n_int, nodes4);
    return cudaGetLastError();
}

// gathers prims in a given order (KD-tree kn order)
__global__ void k_gather_prims(const int32_t *__restrict__ order, int count,
                               const float4 *__restrict__ prims0, float4 *__restrict__ prims) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int s = order[i];
    prims[3 * (size_t)i + 0] = prims0[3 * (size_t)s + 0];
    prims[3 * (size_t)i + 1] = prims0[3 * (size_t)s + 1];
    prims[3 * (size_t)i + 2] = prims0[3 * (size_t)s + 2];
}

// Shape.b / index / morton_code as CLBVH::CLBVH leaves them in the shapes
__global__ void k_export_shapes(const ptgpu_shape *__restrict__ shapes, ptgpu_shape *__restrict__ out,
                                const float *__restrict__ verts, const uint8_t *__restrict__ type,
                                const uint32_t *__restrict__ keys, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float b[6];
    shape_bound(verts, i, type[i] == PTGPU_TRIANGLE, b);
    ptgpu_shape s = shapes[i];
    s.index = i;
    s.morton_code = ~keys[i];
    s.b.min_x = b[0]; s.b.max_x = b[1];
    s.b.min_y = b[2]; s.b.max_y = b[3];
    s.b.min_z = b[4]; s.b.max_z = b[5];
    out[i] = s;
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
static int grid_for(int n, int threads, int cap) {
    int g = (n + threads - 1) / threads;
    return g < 1 ? 1 : (g > cap ? cap : g);
}

cudaError_t launch_unpack_shapes(const ptgpu_shape *d_shapes, int n, float *verts, uint8_t *type,
                                 float4 *prims, Material *mats, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_unpack_shapes<<<(n + 255) / 256, 256, 0, s>>>(d_shapes, n, verts, type, prims, mats);
    return cudaGetLastError();
}

size_t sort_status_words(int n) {
    size_t tiles = ((size_t)n + kSortTile - 1) / kSortTile;
    return tiles * 256 * 5;
}

// block bounds of the emission: in the single-tree build the 256-leaf
// windows' bounds, then the climb's levels above 2^16 leaves; in the batched
// build the levels above the 1024-leaf tiles -- the former needs more, so
// both size by it
size_t block_bound_count(int n) {
    const size_t nblocks = ((size_t)n + kEmitLeaves - 1) / kEmitLeaves;
    return 2 * nblocks + 64;
}

template <class K> static void sort_attrs(K k, size_t smem) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

// A launch that may start before the previous kernel on the stream ends
// (programmatic stream serialisation); the kernel's pdl_begin() waits.
template <typename... P, typename... A>
static cudaError_t launch_chained(void (*k)(P...), int grid, int block, size_t smem, cudaStream_t s,
                                  A... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = PTGPU_PDL;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

// shared-memory opt-ins of the build kernels, once per device; contexts,
// batches, the server's worker and the no-allocation entry point may build
// from different host threads at once, so the per-device flags are guarded
static cudaError_t launch_lbvh_prepare_attrs() {
    static std::mutex attr_mutex;
    static bool attr_set[64] = {false};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(attr_mutex);
    if (dev >= 0 && dev < 64 && attr_set[dev]) return cudaSuccess;
    const size_t smem = sizeof(SortSmem);
    sort_attrs(k_onesweep<true, false>, smem);
    sort_attrs(k_onesweep<false, false>, smem);
    sort_attrs(k_onesweep<false, true>, smem);
    sort_attrs(k_onesweep<false, true, true>, smem);
    cudaFuncSetAttribute(k_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmem);
    cudaFuncSetAttribute(k_tiles_seg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmem);
    e = cudaGetLastError();
    if (e == cudaSuccess && dev >= 0 && dev < 64) attr_set[dev] = true;
    return e;
}

cudaError_t launch_lbvh_build(const LbvhBuffers &b, int n, int all_tri, int sm_count,
                              cudaStream_t s) {
    if (n < 1) return cudaErrorInvalidValue;
    const int ntiles_sort = (n + kSortTile - 1) / kSortTile;
    const int nblocks = (n + kEmitLeaves - 1) / kEmitLeaves;
    cudaError_t e = launch_lbvh_prepare_attrs();
    if (e != cudaSuccess) return e;
    const size_t smem = sizeof(SortSmem);
    // status words: a multiple of 4 (tiles * 256 * 5), cleared as 16-byte words
    if (reinterpret_cast<uintptr_t>(b.status) & 15) return cudaErrorInvalidValue;
    k_init_build<<<sm_count * 2, 256, 0, s>>>(b.state, reinterpret_cast<uint4 *>(b.status),
                                              sort_status_words(n) / 4, b.arrivals, block_bound_count(n),
                                              b.wait_limit);
    const int red_grid = grid_for(n, 256, sm_count * 8);
    e = launch_chained(k_centroid_bounds, red_grid, 256, 0, s, (const float *)b.verts, (const uint8_t *)b.type,
                       all_tri, n, b.state, b.aabbs);
    if (e != cudaSuccess) return e;
#ifndef PTGPU_MORTON_HIST
#define PTGPU_MORTON_HIST 1
#endif
    if (PTGPU_MORTON_HIST) {
        e = launch_chained(k_morton<true>, red_grid, 256, 0, s, (const float *)b.verts, (const float4 *)b.aabbs,
                           (const uint8_t *)b.type, all_tri, n, b.state, b.keys);
        if (e != cudaSuccess) return e;
    } else {
        e = launch_chained(k_morton<false>, red_grid, 256, 0, s, (const float *)b.verts, (const float4 *)b.aabbs,
                           (const uint8_t *)b.type, all_tri, n, b.state, b.keys);
        if (e != cudaSuccess) return e;
        e = launch_chained(k_hist4, grid_for((n + kHistItems - 1) / kHistItems, 256, sm_count * 4), 256, 0, s,
                           (const uint32_t *)b.keys, n, b.state);
        if (e != cudaSuccess) return e;
    }
    const size_t pass_words = (size_t)ntiles_sort * 256;
    const int32_t *no_seg = nullptr;
    // pass 0: keys -> (keys_alt, vals_alt); 1: alt -> tmp; 2: tmp -> alt; 3: alt -> sorted
    e = launch_chained(k_onesweep<true, false>, ntiles_sort, kSortThreads, smem, s, (const uint32_t *)b.keys,
                       (const int32_t *)nullptr, b.keys_alt, b.vals_alt, n, 0, b.state, b.status, no_seg, 0);
    if (e != cudaSuccess) return e;
    e = launch_chained(k_onesweep<false, false>, ntiles_sort, kSortThreads, smem, s,
                       (const uint32_t *)b.keys_alt, (const int32_t *)b.vals_alt, b.keys_tmp, b.vals_tmp, n, 1,
                       b.state, b.status + pass_words, no_seg, 0);
    if (e != cudaSuccess) return e;
    e = launch_chained(k_onesweep<false, false>, ntiles_sort, kSortThreads, smem, s,
                       (const uint32_t *)b.keys_tmp, (const int32_t *)b.vals_tmp, b.keys_alt, b.vals_alt, n, 2,
                       b.state, b.status + 2 * pass_words, no_seg, 0);
    if (e != cudaSuccess) return e;
    e = launch_chained(k_onesweep<false, true>, ntiles_sort, kSortThreads, smem, s,
                       (const uint32_t *)b.keys_alt, (const int32_t *)b.vals_alt, (uint32_t *)nullptr, b.sorted,
                       n, 3, b.state, b.status + 3 * pass_words, no_seg, 0);
    if (e != cudaSuccess) return e;
    // window bounds first in block_bounds, then the climb's levels from 2^16 up
    const int nsuper = (nblocks + 255) / 256;
    e = launch_chained(k_emit, min(nblocks, sm_count * PTGPU_EMIT_MINBLOCKS), kLeafThreads, 0, s,
                       (const float4 *)b.aabbs, (const int32_t *)b.sorted, n, b.btl, b.btn, b.block_bounds,
                       nblocks);
    if (e != cudaSuccess) return e;
    if (nblocks > 1)
        e = launch_chained(k_emit_upper, nsuper, 256, 0, s, (const float *)b.block_bounds, nblocks, n, b.btn,
                           b.block_bounds + 6 * (size_t)nblocks, b.arrivals, nsuper);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

size_t seg_block_bound_count(int n) { return block_bound_count(n); }
int emission_tiles(int n) { return (n + kTileLeaves - 1) / kTileLeaves; }

// The batched build: keys per segment, one radix sort of all keys (four key
// passes, then the segment pass that regroups the shapes by segment while
// keeping each segment's key order -- the order a separate sort of each
// segment gives), and every segment's tiles in one launch.
cudaError_t launch_lbvh_build_seg(const LbvhBuffers &b, int n, const SegBuild &sb, int sm_count,
                                  cudaStream_t s) {
    if (n < 2 || sb.n_segs < 1 || sb.n_segs > kMaxSegments) return cudaErrorInvalidValue;
    cudaError_t e = launch_lbvh_prepare_attrs();
    if (e != cudaSuccess) return e;
    const int ntiles_sort = (n + kSortTile - 1) / kSortTile;
    const size_t smem = sizeof(SortSmem);
    k_init_state<<<1, 256, 0, s>>>(b.state, b.wait_limit);
    k_seg_init<<<(sb.n_segs + 127) / 128, 128, 0, s>>>(sb.seg_state, sb.n_segs, b.state, sb.seg_off);
    e = cudaMemsetAsync(b.status, 0, sort_status_words(n) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(b.arrivals, 0, (size_t)sb.n_blocks * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const int red_grid = grid_for(n, 256, sm_count * 8);
    k_seg_centroid_bounds<<<red_grid, 256, 0, s>>>(b.verts, b.type, n, sb, b.aabbs);
    k_seg_morton<<<red_grid, 256, 0, s>>>(b.verts, b.aabbs, b.type, n, sb, b.keys);
    k_hist4<<<grid_for((n + kHistItems - 1) / kHistItems, 256, sm_count * 4), 256, 0, s>>>(b.keys, n, b.state);
    const size_t pw = (size_t)ntiles_sort * 256;
    // keys -> alt -> tmp -> alt -> tmp, then the segment pass tmp -> sorted
    k_onesweep<true, false><<<ntiles_sort, kSortThreads, smem, s>>>(
        b.keys, nullptr, b.keys_alt, b.vals_alt, n, 0, b.state, b.status);
    k_onesweep<false, false><<<ntiles_sort, kSortThreads, smem, s>>>(
        b.keys_alt, b.vals_alt, b.keys_tmp, b.vals_tmp, n, 1, b.state, b.status + pw);
    k_onesweep<false, false><<<ntiles_sort, kSortThreads, smem, s>>>(
        b.keys_tmp, b.vals_tmp, b.keys_alt, b.vals_alt, n, 2, b.state, b.status + 2 * pw);
    k_onesweep<false, false><<<ntiles_sort, kSortThreads, smem, s>>>(
        b.keys_alt, b.vals_alt, b.keys_tmp, b.vals_tmp, n, 3, b.state, b.status + 3 * pw);
    k_onesweep<false, true, true><<<ntiles_sort, kSortThreads, smem, s>>>(
        nullptr, b.vals_tmp, nullptr, b.sorted, n, 4, b.state, b.status + 4 * pw, sb.seg_off, sb.n_segs);
    k_leaves<<<(n + kLeafThreads - 1) / kLeafThreads, kLeafThreads, 0, s>>>(b.aabbs, b.sorted, n, sb.seg_off,
                                                                             sb.n_segs, b.btl, b.leaf_bounds);
    k_tiles_seg<<<sb.n_tiles, kTileThreads, kTileSmem, s>>>(b.leaf_bounds, sb, b.btn, b.block_bounds,
                                                            b.arrivals);
    return cudaGetLastError();
}

cudaError_t launch_abi_to_trace(const ptgpu_bvh_node *btn, const ptgpu_bvh_node *btl, int n,
                                const float4 *prims0, float4 *nodes, float4 *prims,
                                int32_t *prim_id, cudaStream_t s, int node_base, int shape_base) {
    if (n <= 0) return cudaSuccess;
    k_abi_to_trace<<<(n + 255) / 256, 256, 0, s>>>(btn, btl, n, prims0, nodes, prims, prim_id,
                                                    node_base, shape_base);
    return cudaGetLastError();
}

cudaError_t launch_gather_prims(const int32_t *order, int count, const float4 *prims0,
                                float4 *prims, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    k_gather_prims<<<(count + 255) / 256, 256, 0, s>>>(order, count, prims0, prims);
    return cudaGetLastError();
}

cudaError_t launch_export_shapes(const ptgpu_shape *shapes, ptgpu_shape *out, const float *verts,
                                 const uint8_t *type, const uint32_t *keys, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_export_shapes<<<(n + 255) / 256, 256, 0, s>>>(shapes, out, verts, type, keys, n);
    return cudaGetLastError();
}

}  // namespace ptgpu
