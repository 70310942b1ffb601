// device.cuh -- device-side math and data layouts shared by the kernels.
//
// Float semantics: the library is compiled with -fmad=false and IEEE
// division/square root, so every expression below rounds exactly like the
// reference's OpenCL C (rendering_kernel.cl) evaluated without contraction.
// The helpers are written operand-for-operand in the reference's order.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/ptgpu.h"
#include "types.h"

namespace ptgpu {

constexpr float kEps = 0.01f;                       // EPSILON, geom.h:29
constexpr float kPi = 3.14159265358979323846f;      // FLOAT_PI, geom.h:30
constexpr float kInfT = 1e20f;                      // Intersect's initial t
#ifndef PTGPU_STACK
#define PTGPU_STACK 64
#endif
constexpr int kStackSize = PTGPU_STACK;             // traversal stack entries

struct f3 { float x, y, z; };

__host__ __device__ __forceinline__ f3 mk3(float x, float y, float z) { f3 v; v.x = x; v.y = y; v.z = z; return v; }
__host__ __device__ __forceinline__ f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ f3 mul3(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ f3 smul3(float k, f3 b) { return mk3(k * b.x, k * b.y, k * b.z); }
__host__ __device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ f3 cross3(f3 a, f3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// vnorm (vec.h:41): 1.f / sqrt(dot) then scale
__device__ __forceinline__ f3 norm3(f3 v) { float l = 1.f / sqrtf(dot3(v, v)); return smul3(l, v); }
__host__ __device__ __forceinline__ bool iszero3(f3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }
// OpenCL sign(): +-1, the signed zero itself, 0 for NaN
__device__ __forceinline__ float cl_sign(float x) {
    return x > 0.f ? 1.f : (x < 0.f ? -1.f : (x == x ? x : 0.f));
}
__device__ __forceinline__ float cl_clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
// ternary min/max of AccelCommon.h:14-32 and BVH.cl:78-86 (bounds)
__host__ __device__ __forceinline__ float min2f(float a, float b) { return (a < b) ? a : b; }
__host__ __device__ __forceinline__ float max2f(float a, float b) { return (a > b) ? a : b; }


/* Deterministic sine/cosine used by the GPU library for the light-sphere and
 * diffuse-bounce angles (arguments in [0, 2*pi)).  Quadrant q = round(x*2/pi);
 * three-part Cody-Waite reduction r = x - q*pi/2 with pi/2 split as
 * 1.5703125 (8 significant bits, so q*C1 is exact) + 4.83826792e-4 +
 * 2.56334407e-12; then the Taylor series of sin to r^9 and cos to r^10 on
 * [-pi/4, pi/4] (truncation error below 1e-9).  Plain multiplies and adds
 * in a fixed order, so a CPU build without contraction and the GPU build
 * (-fmad=false) give identical bits. */
#define PT_SINCOS_BODY                                                          \
    float q = floorf(x * 0.636619747f + 0.5f);                                  \
    float r = ((x - q * 1.5703125f) - q * 4.83826792e-4f) - q * 2.56334407e-12f; \
    float r2 = r * r;                                                           \
    float sp = r + r * r2 * (-0.166666672f + r2 * (0.00833333377f +             \
               r2 * (-0.000198412701f + r2 * 2.75573188e-06f)));                \
    float cp = 1.f + r2 * (-0.5f + r2 * (0.0416666679f + r2 * (-0.00138888892f + \
               r2 * (2.48015876e-05f + r2 * -2.75573200e-07f))));               \
    int qi = ((int)q) & 3;                                                      \
    float sv = (qi == 0) ? sp : (qi == 1) ? cp : (qi == 2) ? -sp : -cp;          \
    float cv = (qi == 0) ? cp : (qi == 1) ? -sp : (qi == 2) ? -cp : sp;
__device__ __forceinline__ void pt_sincos(float x, float &s, float &c) {
    PT_SINCOS_BODY
    s = sv;
    c = cv;
}

// GetRandom (rendering_kernel.cl:4-17, simplernd.h:35-49)
__device__ __forceinline__ float get_random(uint32_t &s0, uint32_t &s1) {
    s0 = 36969u * (s0 & 65535u) + (s0 >> 16);
    s1 = 18000u * (s1 & 65535u) + (s1 >> 16);
    uint32_t ires = (s0 << 16) + s1;
    float f = __uint_as_float((ires & 0x007fffffu) | 0x40000000u);
    return (f - 2.f) / 2.f;
}

__device__ __forceinline__ float tri_intersect(f3 p1, f3 e1, f3 e2, f3 o, f3 d) {
    f3 pvec = cross3(d, e2);
    float det = dot3(e1, pvec);
    if (det == 0.f) return 0.f;
    float inv_det = 1.f / det;
    f3 tvec = sub3(o, p1);
    float u = dot3(tvec, pvec) * inv_det;
    if (u < 0.f || u > 1.f) return 0.f;
    f3 qvec = cross3(tvec, e1);
    float v = dot3(d, qvec) * inv_det;
    if (v < 0.f || u + v > 1.f) return 0.f;
    float t = dot3(e2, qvec) * inv_det;
    return t > kEps ? t : 0.f;
}

__device__ __forceinline__ float sphere_intersect(f3 p, float rad2, f3 o, f3 d) {
    f3 op = sub3(p, o);
    float b = dot3(op, d);
    float det = b * b - dot3(op, op) + rad2;
    if (det < 0.f) return 0.f;
    det = sqrtf(det);
    float t = b - det;
    if (t > kEps) return t;
    t = b + det;
    if (t > kEps) return t;
    return 0.f;
}

__device__ __forceinline__ float prim_intersect(const float4 *prims, int k, f3 o, f3 d) {
    float4 a = __ldg(&prims[3 * k + 0]);
    float4 b = __ldg(&prims[3 * k + 1]);
    if (__float_as_int(a.w) == PTGPU_TRIANGLE) {
        float4 c = __ldg(&prims[3 * k + 2]);
        return tri_intersect(mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), mk3(c.x, c.y, c.z), o, d);
    }
    return sphere_intersect(mk3(a.x, a.y, a.z), b.x, o, d);
}

// intersection_bound_test (rendering_kernel.cl:140-192) on one box, with the
// reciprocal direction precomputed (1.0/d rounded to float == 1.f/d).
__device__ __forceinline__ bool slab(float bminx, float bmaxx, float bminy, float bmaxy,
                                     float bminz, float bmaxz, f3 o, f3 inv, float &tmin,
                                     float &tmax) {
    float txmin, txmax, tymin, tymax, tzmin, tzmax;
    if (inv.x >= 0) { txmin = (bminx - o.x) * inv.x; txmax = (bmaxx - o.x) * inv.x; }
    else            { txmin = (bmaxx - o.x) * inv.x; txmax = (bminx - o.x) * inv.x; }
    if (inv.y >= 0) { tymin = (bminy - o.y) * inv.y; tymax = (bmaxy - o.y) * inv.y; }
    else            { tymin = (bmaxy - o.y) * inv.y; tymax = (bminy - o.y) * inv.y; }
    if (inv.z >= 0) { tzmin = (bminz - o.z) * inv.z; tzmax = (bmaxz - o.z) * inv.z; }
    else            { tzmin = (bmaxz - o.z) * inv.z; tzmax = (bminz - o.z) * inv.z; }
    tmin = fmaxf(txmin, fmaxf(tymin, tzmin));
    tmax = fminf(txmax, fminf(tymax, tzmax));
    return tmin <= tmax;
}

// A box is entered when the reference's test passes and it can still hold a
// hit that improves on tbest: entry below tbest (with a 1e-4 relative margin
// for rounding) and exit in front of the origin.
__device__ __forceinline__ bool enter_box(bool hit, float tmin, float tmax, float tbest) {
    return hit && tmin <= tbest * 1.0001f && tmax >= 0.f;
}

// ---------------------------------------------------------------------------
// Ray queries.  One traversal routine serves the closest-hit query
// (Intersect, rendering_kernel.cl:194-363) and the shadow query (IntersectP,
// rendering_kernel.cl:375-395: any hit with 0 < d < maxt, the last shape never
// tested), so a kernel that issues both has a single copy of the loop.
// Boxes are tested with intersection_bound_test's arithmetic; a box is
// entered when that test passes and it can still hold a better hit (front to
// back, nearest child first).  WIDE selects the 4-wide nodes.  COUNT adds
// node visits (v) and primitive tests (p) to *cnt (the benchmark's
// bytes-moved model).
// ---------------------------------------------------------------------------
struct Counts { uint32_t v, p; };

struct Node4 {
    float4 q[8];
};

__device__ __forceinline__ float f4get(const float4 &v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}
__device__ __forceinline__ int i4get(const float4 &v, int k) { return __float_as_int(f4get(v, k)); }

// ---------------------------------------------------------------------------
// Traversal stacks.  LocalStack keeps all of a lane's entries in a local
// array.  ShortStack keeps the bottom SHORT entries in shared memory and only
// the deeper ones in a local array: entry j of lane t sits at
// s[j * LANES + t], so a lane always uses its own bank (LANES is a multiple of
// 32) whatever depth the other lanes are at, and a traversal that stays
// within SHORT entries -- nearly every one in a front-to-back walk -- never
// touches local memory.  Both hold at most STACK entries.
// ---------------------------------------------------------------------------
template <int STACK>
struct LocalStack {
    int loc[STACK];
    __device__ __forceinline__ void put(int i, int v) { loc[i] = v; }
    __device__ __forceinline__ int get(int i) const { return loc[i]; }
};

template <int STACK, int SHORT, int LANES>
struct ShortStack {
    static_assert(SHORT > 0 && SHORT < STACK && LANES % 32 == 0, "short stack shape");
    int *sh;                        // &shared[0][lane of the block]
    int loc[STACK - SHORT];
    __device__ __forceinline__ void put(int i, int v) {
        if (i < SHORT) sh[i * LANES] = v;
        else loc[i - SHORT] = v;
    }
    __device__ __forceinline__ int get(int i) const { return i < SHORT ? sh[i * LANES] : loc[i - SHORT]; }
};

// entries of a lane's stack kept in shared memory (0: all in local memory):
// the closest-hit kernel (2^24 random rays against 4M triangles: 20.68 ->
// 18.74 ms with 16) and the lane tracer (0: 8 / 16 / 24 entries measured
// 29.2 / 29.3 / 29.4 against 28.8 ms per benchmark frame -- the shared
// memory they take comes out of the L1 that caches the scene's nodes)
#ifndef PTGPU_SHORT_STACK
#define PTGPU_SHORT_STACK 16
#endif
#ifndef PTGPU_RENDER_SHORT_STACK
#define PTGPU_RENDER_SHORT_STACK 0
#endif

// A query in flight: the ray, the best hit so far and the traversal
// position (current item and stack depth; the stack itself is the caller's).
// trav_begin sets it up, trav_step advances it by one item, so a kernel can
// interleave the queries of its lanes with other work between steps.
struct Trav {
    f3 o, d, inv;
    float tb;      // closest: best t so far; shadow: maxt
    int prim;      // closest: traversal-order index of the best hit
    int cur, ccnt; // current item: internal node (ccnt == 0) or leaf range
    int sp;
    int any, hit;  // shadow query; a hit was found (shadow: occluded).  In the
                   // BVH and KD walks any intersection sets it, recorded or not
                   // (rendering_kernel.cl `intersected = 1`); brute force: t < inf
};

// Where a query starts: the root item, the scene's shape count and the shape
// IntersectP never tests (its last one).  A batched render keeps the nodes and
// primitives of all its scenes in shared arrays and starts each query at its
// scene's root.
struct TraceRoot {
    int32_t first, count;   // internal node `first` (count 0) or a leaf range
    int32_t n_shapes;
    int32_t skip;           // prim_id value of the scene's last shape
    const float *box;       // min_x,max_x,min_y,max_y,min_z,max_z of the root
};

__device__ __forceinline__ TraceRoot view_root(const TraceView &tv) {
    TraceRoot r;
    r.first = tv.root_count > 0 ? tv.root_first : 0;
    r.count = tv.root_count > 0 ? tv.root_count : 0;
    r.n_shapes = tv.n_shapes;
    r.skip = tv.n_shapes - 1;
    r.box = tv.root_box;
    return r;
}

// Starts a query.  Returns true when it is already answered (empty scene,
// brute-force mode, or the root box missed).
template <bool COUNT>
__device__ __forceinline__ bool trav_begin(const TraceView &tv, const TraceRoot &root, Trav &q,
                                           f3 o, f3 d, bool any, float maxt, Counts *cnt) {
    q.o = o;
    q.d = d;
    q.any = any;
    q.hit = 0;
    q.prim = -1;
    q.tb = any ? maxt : kInfT;
    q.sp = 0;
    const int n = root.n_shapes;
    if (n <= 0 || (any && n <= 1)) return true;
    if (tv.accel == PTGPU_ACCEL_NONE) {
        if (any) {
            for (int i = n - 2; i >= 0; --i) {
                float dd = prim_intersect(tv.prims, i, o, d);
                if (COUNT) cnt->p++;
                if (dd != 0.f && dd < maxt) { q.hit = 1; return true; }
            }
            return true;
        }
        for (int i = n - 1; i >= 0; --i) {
            float dd = prim_intersect(tv.prims, i, o, d);
            if (COUNT) cnt->p++;
            if (dd != 0.f && dd < q.tb) { q.tb = dd; q.prim = i; }
        }
        q.hit = q.tb < kInfT;
        return true;
    }
    q.inv = mk3(1.f / d.x, 1.f / d.y, 1.f / d.z);
    float tmin, tmax;
    if (!slab(__ldg(root.box + 0), __ldg(root.box + 1), __ldg(root.box + 2), __ldg(root.box + 3),
              __ldg(root.box + 4), __ldg(root.box + 5), o, q.inv, tmin, tmax))
        return true;
    q.cur = root.first;
    q.ccnt = root.count;
    return false;
}

template <bool COUNT>
__device__ __forceinline__ bool trav_begin(const TraceView &tv, Trav &q, f3 o, f3 d, bool any,
                                           float maxt, Counts *cnt) {
    return trav_begin<COUNT>(tv, view_root(tv), q, o, d, any, maxt, cnt);
}

// One item of the traversal: a leaf range's primitives or one node's
// children.  Returns true when the query is answered.  skip: the prim_id a
// shadow query never tests (the scene's last shape, TraceRoot::skip).
#ifndef PTGPU_TRAV_FUSE
#define PTGPU_TRAV_FUSE 1
#endif
template <bool WIDE, bool COUNT, int STACK = kStackSize, class Stack>
__device__ __forceinline__ bool trav_step(const TraceView &tv, Trav &q, Stack &stack, Counts *cnt, int skip) {
    if (q.ccnt > 0) {
        for (int k = q.cur; k < q.cur + q.ccnt; ++k) {
            if (q.any && __ldg(&tv.prim_id[k]) == skip) continue;
            float dd = prim_intersect(tv.prims, k, q.o, q.d);
            if (COUNT) cnt->p++;
            if (dd != 0.f) {
                if (q.any) {
                    if (dd < q.tb) { q.hit = 1; return true; }
                } else {
                    q.hit = 1;
                    // equal t: the lower traversal-order index wins, which in
                    // the BVH is the leaf the reference's left-first walk
                    // meets first (its `d < t` keeps the first one found)
                    if (dd < q.tb || (dd == q.tb && k < q.prim)) { q.tb = dd; q.prim = k; }
                }
            }
        }
        if (q.sp == 0) return true;
        int e = stack.get(--q.sp);
        if (e < 0) { q.cur = ~e; q.ccnt = stack.get(--q.sp); }
        else { q.cur = e; q.ccnt = 0; }
        // a node popped after a leaf is visited in the same step, so lanes
        // at a leaf and lanes at a node share the node half of the step
        if (!PTGPU_TRAV_FUSE || q.ccnt > 0) return false;
    }
    if (WIDE) {
        const float4 *p = tv.nodes4 + 8 * (size_t)q.cur;
        Node4 nd;
#pragma unroll
        for (int k = 0; k < 8; ++k) nd.q[k] = __ldg(p + k);
        if (COUNT) cnt->v++;
        // hit children: leaves first in slot order, then internal nodes by distance
        int iref[4];
        float idist[4];
        int ni = 0;
        int lref[4], lcnt[4];
        int nl = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = i4get(nd.q[7], k);
            float t0, t1;
            bool h = slab(f4get(nd.q[0], k), f4get(nd.q[1], k), f4get(nd.q[2], k),
                          f4get(nd.q[3], k), f4get(nd.q[4], k), f4get(nd.q[5], k), q.o, q.inv, t0,
                          t1);
            if (c < 0 || !enter_box(h, t0, t1, q.tb)) continue;
            if (c > 0) { lref[nl] = i4get(nd.q[6], k); lcnt[nl] = c; ++nl; }
            else { iref[ni] = i4get(nd.q[6], k); idist[ni] = t0; ++ni; }
        }
        // internal children: sort nearest first, push the others far first
#pragma unroll
        for (int a = 1; a < 4; ++a) {
            if (a < ni) {
                float dv = idist[a];
                int rv = iref[a];
                int b = a - 1;
                while (b >= 0 && idist[b] > dv) { idist[b + 1] = idist[b]; iref[b + 1] = iref[b]; --b; }
                idist[b + 1] = dv;
                iref[b + 1] = rv;
            }
        }
        for (int a = ni - 1; a >= 0; --a) {
            if (q.sp < STACK) stack.put(q.sp++, iref[a]);
            else if (tv.error_flags) atomicOr(tv.error_flags, 1);
        }
        // leaves go on the stack as negative entries, tested before the nodes
        for (int a = nl - 1; a >= 0; --a) {
            if (q.sp + 1 < STACK) { stack.put(q.sp++, lcnt[a]); stack.put(q.sp++, ~lref[a]); }
            else if (tv.error_flags) atomicOr(tv.error_flags, 1);
        }
    } else {
        const float4 *nd = tv.nodes + 4 * (size_t)q.cur;
        float4 q0 = __ldg(nd + 0), q1 = __ldg(nd + 1), q2 = __ldg(nd + 2);
        int4 q3 = __ldg(reinterpret_cast<const int4 *>(nd + 3));
        if (COUNT) cnt->v++;
        float lt0, lt1, rt0, rt1;
        bool lh = slab(q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q.o, q.inv, lt0, lt1);
        bool rh = slab(q1.z, q1.w, q2.x, q2.y, q2.z, q2.w, q.o, q.inv, rt0, rt1);
        lh = enter_box(lh, lt0, lt1, q.tb);
        rh = enter_box(rh, rt0, rt1, q.tb);
        if (lh && rh) {
            // nearer child next, the other onto the stack (leaf: negative pair)
            bool lfirst = !(rt0 < lt0);
            int fr = lfirst ? q3.y : q3.x, fc = lfirst ? q3.w : q3.z;
            int nr = lfirst ? q3.x : q3.y, nc = lfirst ? q3.z : q3.w;
            if (q.sp + 1 < STACK) {
                if (fc > 0) { stack.put(q.sp++, fc); stack.put(q.sp++, ~fr); }
                else stack.put(q.sp++, fr);
            } else if (tv.error_flags) atomicOr(tv.error_flags, 1);
            q.cur = nr; q.ccnt = nc;
            return false;
        }
        if (lh) { q.cur = q3.x; q.ccnt = q3.z; return false; }
        if (rh) { q.cur = q3.y; q.ccnt = q3.w; return false; }
    }
    if (q.sp == 0) return true;
    int e = stack.get(--q.sp);
    if (e < 0) { q.cur = ~e; q.ccnt = stack.get(--q.sp); }
    else { q.cur = e; q.ccnt = 0; }
    return false;
}

// A whole query.  Returns: closest query -> the reference's `intersected`
// (t, prim set); shadow query -> 1 when occluded.
template <bool WIDE, bool COUNT>
__device__ __forceinline__ int trace_query(const TraceView &tv, f3 o, f3 d, bool any, float maxt,
                                           float &t, int &prim, Counts *cnt) {
    Trav q;
    LocalStack<kStackSize> stack;
    if (!trav_begin<COUNT>(tv, q, o, d, any, maxt, cnt))
        while (!trav_step<WIDE, COUNT>(tv, q, stack, cnt, tv.n_shapes - 1)) {}
    t = any ? kInfT : q.tb;
    prim = q.prim;
    return q.hit;
}

}  // namespace ptgpu
