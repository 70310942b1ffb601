// lbvh.cu -- GPU LBVH build for the reference BVH layout (CLBVH + BVH.cl).
//
// Pipeline (reference mode, all on one stream):
//   k_centroid_bounds   centroid min/max over all shapes (CLBVH.cpp:91-123)
//   k_morton_hist       30-bit Morton keys (CLBVH.cpp:125-164) + the digit
//                       histograms of all four radix passes
//   k_onesweep x4       stable LSD radix sort of ~key (== the descending
//                       stable bubble sort, CLBVH.cpp:31-47), 8-bit digits,
//                       warp-level ranking, decoupled look-back with a
//                       bounded spin
//   k_tiles             per 1024-leaf tile: leaf records + every internal node
//                       inside the tile, bounds by an in-shared-memory
//                       bottom-up reduction (kernelConstructRadixTree and
//                       kernelConstructBVHTree, BVH.cl:141-258, with the
//                       closed-form topology of lbvh_topo.cuh)
//   k_top               the internal nodes above the tiles
// The result is the reference's btn[N-1]/btl[N] arrays, resident on the
// device.  k_abi_to_trace then derives the 64-byte traversal nodes.
#include <cfloat>
#include <cstring>
#include <cstdint>
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

__global__ void k_init_state(BuildState *st) {
    int t = threadIdx.x;
    for (int i = t; i < 4 * 256; i += blockDim.x) (&st->hist[0][0])[i] = 0u;
    if (t < 4) st->tile_counter[t] = 0u;
    if (t == 0) {
        st->error = 0u;
        st->top_ticket = 0u;
        // the reference's initial values: FLT_MAX for minima, FLT_MIN for maxima
        for (int a = 0; a < 3; ++a) {
            st->cmin[a] = f2ord(FLT_MAX);
            st->cmax[a] = f2ord(FLT_MIN);
        }
    }
}

__global__ void __launch_bounds__(256) k_centroid_bounds(const float *__restrict__ verts,
                                                          const uint8_t *__restrict__ type,
                                                          int all_tri, int n, BuildState *st) {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        bool tri = all_tri || type[i] == PTGPU_TRIANGLE;
        f3 p = shape_centroid(verts, i, tri);
        float c[3] = {p.x, p.y, p.z};
        for (int a = 0; a < 3; ++a) {
            if (c[a] == c[a]) {          // NaN centroids never pass the reference's < / >
                lo[a] = fminf(lo[a], c[a]);
                hi[a] = fmaxf(hi[a], c[a]);
            }
        }
    }
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    __shared__ float s_lo[8][3], s_hi[8][3];
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) for (int a = 0; a < 3; ++a) { s_lo[w][a] = lo[a]; s_hi[w][a] = hi[a]; }
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

__device__ __forceinline__ uint32_t morton30(uint32_t a, uint32_t b, uint32_t c) {
    // bit j of a (j = 9..0) goes to 3j+2, of b to 3j+1, of c to 3j (CLBVH.cpp:158-163)
    uint32_t code = 0;
#pragma unroll
    for (int j = 0; j < 10; ++j) {
        code |= ((a >> j) & 1u) << (3 * j + 2);
        code |= ((b >> j) & 1u) << (3 * j + 1);
        code |= ((c >> j) & 1u) << (3 * j + 0);
    }
    return code;
}

// Morton keys + per-pass digit histograms.  The sort key is ~code so an
// ascending stable sort gives the reference's descending stable order.
__global__ void __launch_bounds__(256) k_morton_hist(const float *__restrict__ verts,
                                                      const uint8_t *__restrict__ type,
                                                      int all_tri, int n, BuildState *st,
                                                      uint32_t *__restrict__ keys) {
    __shared__ uint32_t s_hist[4][256];
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) (&s_hist[0][0])[i] = 0u;
    __syncthreads();
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) { lo[a] = ord2f(st->cmin[a]); hi[a] = ord2f(st->cmax[a]); }
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        int i = base + threadIdx.x;
        bool valid = i < n;
        uint32_t key = 0;
        if (valid) {
            bool tri = all_tri || type[i] == PTGPU_TRIANGLE;
            f3 p = shape_centroid(verts, i, tri);
            uint32_t qa = quantise10(p.x, lo[0], hi[0]);
            uint32_t qb = quantise10(p.y, lo[1], hi[1]);
            uint32_t qc = quantise10(p.z, lo[2], hi[2]);
            key = ~morton30(qa & 1023u, qb & 1023u, qc & 1023u);
            keys[i] = key;
        }
        unsigned vm = __ballot_sync(0xffffffffu, valid);
        if (valid) {
#pragma unroll
            for (int d = 0; d < 4; ++d) {
                uint32_t dig = (key >> (8 * d)) & 255u;
                unsigned peers = __match_any_sync(vm, dig);
                if (lane == __ffs(peers) - 1) atomicAdd(&s_hist[d][dig], (uint32_t)__popc(peers));
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) {
        uint32_t v = (&s_hist[0][0])[i];
        if (v) atomicAdd(&st->hist[0][0] + i, v);
    }
}

// ---------------------------------------------------------------------------
// onesweep radix pass
// ---------------------------------------------------------------------------
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 15;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr uint32_t kFlagAgg = 1u << 30, kFlagInc = 2u << 30, kValMask = (1u << 30) - 1u;
constexpr int kSpinLimit = 1 << 22;

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) {
    return *reinterpret_cast<const volatile uint32_t *>(p);
}
__device__ __forceinline__ void st_volatile(uint32_t *p, uint32_t v) {
    *reinterpret_cast<volatile uint32_t *>(p) = v;
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

struct SortSmem {
    uint32_t warp_hist[kSortWarps][256];
    uint32_t digit_start[256];
    uint32_t tile_excl[256];
    uint32_t scan_tmp[32];
    uint32_t keys[kSortTile];
    int32_t vals[kSortTile];
    int tile;
    int abort;
};

template <bool FIRST, bool LAST>
__global__ void __launch_bounds__(kSortThreads) k_onesweep(const uint32_t *__restrict__ keys_in,
                                                            const int32_t *__restrict__ vals_in,
                                                            uint32_t *__restrict__ keys_out,
                                                            int32_t *__restrict__ vals_out, int n,
                                                            int pass, BuildState *st,
                                                            uint32_t *status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem &sm = *reinterpret_cast<SortSmem *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int shift = 8 * pass;
    if (tid == 0) { sm.tile = (int)atomicAdd(&st->tile_counter[pass], 1u); sm.abort = 0; }
    for (int i = tid; i < kSortWarps * 256; i += kSortThreads) (&sm.warp_hist[0][0])[i] = 0u;
    // global digit offsets for this pass
    uint32_t gcount = st->hist[pass][tid];
    uint32_t goff = block_excl_scan256(gcount, sm.scan_tmp);
    __syncthreads();
    const int tile = sm.tile;
    const int64_t base = (int64_t)tile * kSortTile;
    uint32_t key[kSortItems];
    int32_t val[kSortItems];
    uint32_t rank[kSortItems];
    const unsigned lt_mask = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        int64_t idx = base + (int64_t)w * 32 * kSortItems + j * 32 + lane;
        bool valid = idx < n;
        key[j] = valid ? keys_in[idx] : 0xffffffffu;
        val[j] = valid ? (FIRST ? (int32_t)idx : vals_in[idx]) : -1;
        uint32_t dig = (key[j] >> shift) & 255u;
        unsigned vm = __ballot_sync(0xffffffffu, valid);
        rank[j] = 0xffffffffu;
        if (valid) {
            unsigned peers = __match_any_sync(vm, dig);
            uint32_t prev = sm.warp_hist[w][dig];
            rank[j] = prev + (uint32_t)__popc(peers & lt_mask);
            __syncwarp(peers);
            if (lane == __ffs(peers) - 1) sm.warp_hist[w][dig] = prev + (uint32_t)__popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    // per-digit counts: exclusive prefix over warps, tile total
    uint32_t count = 0;
#pragma unroll
    for (int k = 0; k < kSortWarps; ++k) {
        uint32_t c = sm.warp_hist[k][tid];
        sm.warp_hist[k][tid] = count;
        count += c;
    }
    uint32_t dstart = block_excl_scan256(count, sm.scan_tmp);
    sm.digit_start[tid] = dstart;
    // decoupled look-back, one digit per thread
    uint32_t *my = status + (size_t)tile * 256 + tid;
    uint32_t excl = 0;
    if (tile == 0) {
        st_volatile(my, kFlagInc | count);
    } else {
        st_volatile(my, kFlagAgg | count);
        int p = tile - 1;
        bool timed_out = false;
        while (p >= 0) {
            uint32_t v;
            int spins = 0;
            for (;;) {
                v = ld_volatile(status + (size_t)p * 256 + tid);
                if (v & (3u << 30)) break;
                if (++spins > kSpinLimit) { timed_out = true; break; }
                __nanosleep(32);
            }
            if (timed_out) break;
            excl += v & kValMask;
            if ((v & (3u << 30)) == kFlagInc) break;
            --p;
        }
        if (timed_out) { atomicOr(&st->error, 1u); sm.abort = 1; }
        st_volatile(my, kFlagInc | ((excl + count) & kValMask));
    }
    sm.tile_excl[tid] = goff + excl;
    __syncthreads();
    // scatter into shared memory in tile-sorted order
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        if (rank[j] != 0xffffffffu) {
            uint32_t dig = (key[j] >> shift) & 255u;
            uint32_t pos = sm.digit_start[dig] + sm.warp_hist[w][dig] + rank[j];
            sm.keys[pos] = key[j];
            sm.vals[pos] = val[j];
        }
    }
    __syncthreads();
    if (sm.abort) return;
    const int valid_cnt = (int)min((int64_t)kSortTile, (int64_t)n - base);
    for (int i = tid; i < valid_cnt; i += kSortThreads) {
        uint32_t k = sm.keys[i];
        uint32_t dig = (k >> shift) & 255u;
        uint32_t dest = sm.tile_excl[dig] + ((uint32_t)i - sm.digit_start[dig]);
        if (dest < (uint32_t)n) {
            if (!LAST) keys_out[dest] = k;
            vals_out[dest] = sm.vals[i];
        }
    }
}

// ---------------------------------------------------------------------------
// emission + refit
// ---------------------------------------------------------------------------
constexpr int kTileLeaves = 1024;
constexpr int kTileLog = 10;
constexpr int kTileThreads = 512;

__device__ __forceinline__ void write_node(ptgpu_bvh_node *dst, int mn, int mx, int nshape, int leaf,
                                           int nl, int nr, int np, const float b[6], uint32_t cost_bits,
                                           uint32_t area_bits) {
    int *d = reinterpret_cast<int *>(dst);
    d[0] = mn; d[1] = mx; d[2] = nshape; d[3] = leaf; d[4] = nl; d[5] = nr; d[6] = np;
    float *f = reinterpret_cast<float *>(dst) + 7;
    f[0] = b[0]; f[1] = b[1]; f[2] = b[2]; f[3] = b[3]; f[4] = b[4]; f[5] = b[5];
    d[13] = (int)cost_bits; d[14] = (int)area_bits;
}

__device__ __forceinline__ void merge6(float *a, const float *b) {   // merge_bounds(a, b)
    a[0] = min2f(a[0], b[0]); a[1] = max2f(a[1], b[1]);
    a[2] = min2f(a[2], b[2]); a[3] = max2f(a[3], b[3]);
    a[4] = min2f(a[4], b[4]); a[5] = max2f(a[5], b[5]);
}

// emits the record of the node covering block [lo, hi] (right half non-empty)
__device__ __forceinline__ void emit_internal(ptgpu_bvh_node *btn, int lo, int hi, int level,
                                              int n, const float b[6]) {
    int32_t a_lo, a_hi, a_g;
    topo_range(lo, n, a_lo, a_hi, a_g);
    int idx = (a_lo == lo && a_hi == hi) ? lo : hi;
    if (idx < 0 || idx > n - 2) return;   // unreachable for a valid block; keeps writes in bounds
    int gamma = lo + (1 << (level - 1)) - 1;
    bool ll = (level == 1), rl = (hi == gamma + 1);
    int parent = topo_parent_internal(idx, lo, hi, n);
    write_node(&btn[idx], lo, hi, 0, (ll || rl) ? 2 : 0, gamma, gamma + 1, parent, b, 0u, 0u);
}

__global__ void __launch_bounds__(kTileThreads) k_tiles(const float *__restrict__ verts,
                                                         const uint8_t *__restrict__ type,
                                                         int all_tri, const int32_t *__restrict__ sorted,
                                                         int n, ptgpu_bvh_node *__restrict__ btn,
                                                         ptgpu_bvh_node *__restrict__ btl,
                                                         float *__restrict__ tile_bounds) {
    __shared__ float sb[6][kTileLeaves];
    const int T0 = blockIdx.x * kTileLeaves;
    const int cnt = min(kTileLeaves, n - T0);
    for (int k = threadIdx.x; k < cnt; k += kTileThreads) {
        int leaf = T0 + k;
        int s = min(max(sorted[leaf], 0), n - 1);   // in bounds even after a failed sort
        bool tri = all_tri || type[s] == PTGPU_TRIANGLE;
        float b[6];
        shape_bound(verts, s, tri, b);
        for (int a = 0; a < 6; ++a) sb[a][k] = b[a];
        int parent = n >= 2 ? topo_parent_leaf(leaf, n) : -1;
        write_node(&btl[leaf], -1, -1, s, -1, -1, -1, parent, b, 0xffffffffu, 0xffffffffu);
    }
    __syncthreads();
    for (int level = 1; level <= kTileLog; ++level) {
        const int half = 1 << (level - 1);
        const int nblk = (cnt + (1 << level) - 1) >> level;
        for (int bidx = threadIdx.x; bidx < nblk; bidx += kTileThreads) {
            int l0 = bidx << level;
            int r0 = l0 + half;
            if (r0 < cnt) {
                float b[6], c[6];
                for (int a = 0; a < 6; ++a) { b[a] = sb[a][l0]; c[a] = sb[a][r0]; }
                merge6(b, c);
                for (int a = 0; a < 6; ++a) sb[a][l0] = b[a];
                int lo = T0 + l0;
                int hi = min(T0 + l0 + (1 << level), n) - 1;
                emit_internal(btn, lo, hi, level, n, b);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 6) tile_bounds[(size_t)blockIdx.x * 6 + threadIdx.x] = sb[threadIdx.x][0];
}

// levels above the tiles: one CTA, bounds of tile-aligned blocks kept in
// shared memory (global memory when there are more than kTopSmemTiles tiles)
constexpr int kTopThreads = 1024;
constexpr int kTopSmemTiles = 4096;

__global__ void __launch_bounds__(kTopThreads) k_top(float *__restrict__ tile_bounds, int ntiles,
                                                      int n, ptgpu_bvh_node *__restrict__ btn) {
    extern __shared__ float tb[];   // [ntiles][6] when it fits
    const bool in_smem = ntiles <= kTopSmemTiles;
    float *arr = in_smem ? tb : tile_bounds;
    if (in_smem)
        for (int i = threadIdx.x; i < ntiles * 6; i += kTopThreads) tb[i] = tile_bounds[i];
    __syncthreads();
    for (int level = kTileLog + 1; (1 << (level - 1)) < n; ++level) {
        const int step = 1 << (level - kTileLog);        // tiles per block at this level
        const int halfstep = step >> 1;
        const int nblk = (ntiles + step - 1) / step;
        for (int bidx = threadIdx.x; bidx < nblk; bidx += kTopThreads) {
            int j = bidx * step;
            int jr = j + halfstep;
            if (jr < ntiles) {
                float b[6], c[6];
                for (int a = 0; a < 6; ++a) { b[a] = arr[j * 6 + a]; c[a] = arr[jr * 6 + a]; }
                merge6(b, c);
                for (int a = 0; a < 6; ++a) arr[j * 6 + a] = b[a];
                int lo = j * kTileLeaves;
                int64_t he = (int64_t)lo + ((int64_t)1 << level);
                int hi = (int)((he < n ? he : n) - 1);
                emit_internal(btn, lo, hi, level, n, b);
            }
        }
        if (!in_smem) __threadfence_block();
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// ABI arrays -> traversal layout (works for any btn/btl, including trees
// installed by the caller or restructured by the treelet pass): a child is a
// leaf when nLeft == min / nRight == max.
// ---------------------------------------------------------------------------
__global__ void k_abi_to_trace(const ptgpu_bvh_node *__restrict__ btn,
                               const ptgpu_bvh_node *__restrict__ btl, int n,
                               const float4 *__restrict__ prims0, float4 *__restrict__ nodes,
                               float4 *__restrict__ prims, int32_t *__restrict__ prim_id) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        int s = min(max(btl[i].nShape, 0), n - 1);
        prim_id[i] = s;
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
        int4 q = make_int4(li, ri, ll ? 1 : 0, rl ? 1 : 0);
        o[3] = *reinterpret_cast<float4 *>(&q);
    }
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
__global__ void k_export_shapes(ptgpu_shape *__restrict__ shapes, const float *__restrict__ verts,
                                const uint8_t *__restrict__ type, const uint32_t *__restrict__ keys,
                                int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float b[6];
    shape_bound(verts, i, type[i] == PTGPU_TRIANGLE, b);
    shapes[i].index = i;
    shapes[i].morton_code = ~keys[i];
    shapes[i].b.min_x = b[0]; shapes[i].b.max_x = b[1];
    shapes[i].b.min_y = b[2]; shapes[i].b.max_y = b[3];
    shapes[i].b.min_z = b[4]; shapes[i].b.max_z = b[5];
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
    return tiles * 256 * 4;
}

cudaError_t launch_lbvh_build(const LbvhBuffers &b, int n, int all_tri, int sm_count,
                              cudaStream_t s) {
    if (n < 1) return cudaErrorInvalidValue;
    const int ntiles_sort = (n + kSortTile - 1) / kSortTile;
    cudaError_t e;
    k_init_state<<<1, 256, 0, s>>>(b.state);
    e = cudaMemsetAsync(b.status, 0, sort_status_words(n) * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const int red_grid = grid_for(n, 256, sm_count * 8);
    k_centroid_bounds<<<red_grid, 256, 0, s>>>(b.verts, b.type, all_tri, n, b.state);
    k_morton_hist<<<red_grid, 256, 0, s>>>(b.verts, b.type, all_tri, n, b.state, b.keys);
    const size_t smem = sizeof(SortSmem);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_onesweep<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_onesweep<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_onesweep<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_top, cudaFuncAttributeMaxDynamicSharedMemorySize, kTopSmemTiles * 6 * 4);
        attr_set = true;
    }
    const size_t pass_words = (size_t)ntiles_sort * 256;
    // pass 0: keys -> (keys_alt, vals_alt); 1: alt -> main; 2: main -> alt; 3: alt -> sorted
    k_onesweep<true, false><<<ntiles_sort, kSortThreads, smem, s>>>(
        b.keys, nullptr, b.keys_alt, b.vals_alt, n, 0, b.state, b.status);
    k_onesweep<false, false><<<ntiles_sort, kSortThreads, smem, s>>>(
        b.keys_alt, b.vals_alt, b.keys_tmp, b.vals_tmp, n, 1, b.state, b.status + pass_words);
    k_onesweep<false, false><<<ntiles_sort, kSortThreads, smem, s>>>(
        b.keys_tmp, b.vals_tmp, b.keys_alt, b.vals_alt, n, 2, b.state, b.status + 2 * pass_words);
    k_onesweep<false, true><<<ntiles_sort, kSortThreads, smem, s>>>(
        b.keys_alt, b.vals_alt, nullptr, b.sorted, n, 3, b.state, b.status + 3 * pass_words);
    const int ntiles = (n + kTileLeaves - 1) / kTileLeaves;
    k_tiles<<<ntiles, kTileThreads, 0, s>>>(b.verts, b.type, all_tri, b.sorted, n, b.btn, b.btl,
                                            b.tile_bounds);
    if (ntiles > 1) {
        size_t tsm = ntiles <= kTopSmemTiles ? (size_t)ntiles * 6 * 4 : 0;
        k_top<<<1, kTopThreads, tsm, s>>>(b.tile_bounds, ntiles, n, b.btn);
    }
    return cudaGetLastError();
}

cudaError_t launch_abi_to_trace(const ptgpu_bvh_node *btn, const ptgpu_bvh_node *btl, int n,
                                const float4 *prims0, float4 *nodes, float4 *prims,
                                int32_t *prim_id, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_abi_to_trace<<<(n + 255) / 256, 256, 0, s>>>(btn, btl, n, prims0, nodes, prims, prim_id);
    return cudaGetLastError();
}

cudaError_t launch_gather_prims(const int32_t *order, int count, const float4 *prims0,
                                float4 *prims, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    k_gather_prims<<<(count + 255) / 256, 256, 0, s>>>(order, count, prims0, prims);
    return cudaGetLastError();
}

cudaError_t launch_export_shapes(ptgpu_shape *shapes, const float *verts, const uint8_t *type,
                                 const uint32_t *keys, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_export_shapes<<<(n + 255) / 256, 256, 0, s>>>(shapes, verts, type, keys, n);
    return cudaGetLastError();
}

}  // namespace ptgpu
