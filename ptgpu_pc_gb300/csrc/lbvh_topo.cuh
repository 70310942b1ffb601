// lbvh_topo.cuh -- closed-form topology of the reference LBVH.
//
// kernelConstructRadixTree (BVH.cl:141-208) runs Karras' construction with
// the common prefix taken over the *indices* (longestCommonPrefix compares
// i ^ j, BVH.cl:127-134), so the tree depends only on N: it is the compressed
// binary trie of the integers 0..N-1.  Every node covers an aligned block
// [b*2^h, (b+1)*2^h - 1] clipped to N-1 and splits at its highest differing
// bit; a left child is numbered by its range end, a right child by its range
// start, the root is node 0 (Karras 2012 numbering).  These functions return
// the same min/max/nLeft/nRight/leaf/nParent fields the reference kernel
// writes, from the node index alone, so the build can emit each node record
// once without a top-down pass.  Checked against the reference kernel for
// every N up to a few thousand and for large N by the tests.
#pragma once
#include <cstdint>

namespace ptgpu {

struct TopoNode {
    int32_t lo, hi;      // leaf range (min, max)
    int32_t gamma;       // split: nLeft = gamma, nRight = gamma + 1
    int32_t parent;      // nParent (0 for the root, as the zeroed buffer holds)
    bool left_leaf, right_leaf;
};

__host__ __device__ __forceinline__ int topo_ctz(uint32_t v) {
#ifdef __CUDA_ARCH__
    return __ffs((int)v) - 1;
#else
    return __builtin_ctz(v);
#endif
}
__host__ __device__ __forceinline__ int topo_bits(uint32_t v) {   // 32 - clz(v), v != 0
#ifdef __CUDA_ARCH__
    return 32 - __clz((int)v);
#else
    return 32 - __builtin_clz(v);
#endif
}

// Range and split of internal node i (0 <= i <= n-2, n >= 2).
__host__ __device__ __forceinline__ void topo_range(int32_t i, int32_t n, int32_t &lo,
                                                    int32_t &hi, int32_t &gamma) {
    if (i & 1) {                         // odd: a left child, range ends at i
        int L = topo_ctz((uint32_t)i + 1u);
        lo = i + 1 - (1 << L);
        hi = i;
    } else if (i == 0) {                 // root
        lo = 0;
        hi = n - 1;
    } else {                             // even: a right child, range starts at i
        int h = topo_ctz((uint32_t)i);
        int64_t e = (int64_t)i + ((int64_t)1 << h);
        lo = i;
        hi = (int32_t)((e < (int64_t)n ? e : (int64_t)n) - 1);
    }
    int hb = topo_bits((uint32_t)(lo ^ hi));
    gamma = lo + (1 << (hb - 1)) - 1;
}

// Parent of the node covering [lo, hi] whose index is `self` (internal) --
// either the node numbered lo (when the parent is a right child or the root)
// or the one numbered by the parent's range end (when it is a left child).
__host__ __device__ __forceinline__ int32_t topo_parent_internal(int32_t self, int32_t lo,
                                                                 int32_t hi, int32_t n) {
    if (self == 0) return 0;
    if (self & 1) {
        // left child: parent's split is `self`; candidate A = node lo
        if (lo != self && lo <= n - 2) {
            int32_t a_lo, a_hi, a_g;
            topo_range(lo, n, a_lo, a_hi, a_g);
            if (a_g == self) return lo;
        } else if (lo == 0) {
            int32_t a_lo, a_hi, a_g;
            topo_range(0, n, a_lo, a_hi, a_g);
            if (a_g == self) return 0;
        }
        // otherwise the parent is a complete left child ending at lo + 2*size - 1
        int32_t size = hi - lo + 1;
        return lo + 2 * size - 1;
    }
    // right child: parent's split is self - 1; candidate A = node hi (a left child)
    if ((hi & 1) && hi <= n - 2 && hi != self) {
        int32_t a_lo, a_hi, a_g;
        topo_range(hi, n, a_lo, a_hi, a_g);
        if (a_g == self - 1) return hi;
    }
    int h = topo_ctz((uint32_t)self);
    return self - (1 << h);
}

__host__ __device__ __forceinline__ TopoNode topo_node(int32_t i, int32_t n) {
    TopoNode t;
    topo_range(i, n, t.lo, t.hi, t.gamma);
    t.left_leaf = (t.lo == t.gamma);
    t.right_leaf = (t.hi == t.gamma + 1);
    t.parent = topo_parent_internal(i, t.lo, t.hi, n);
    return t;
}

// Parent of leaf k (0 <= k <= n-1, n >= 2).
__host__ __device__ __forceinline__ int32_t topo_parent_leaf(int32_t k, int32_t n) {
    if ((k & 1) == 0) {
        if (k + 1 <= n - 1) {
            // the 2-leaf block [k, k+1] is a node: index k+1 if it is a left child
            if (k + 1 <= n - 2) {
                int32_t lo, hi, g;
                topo_range(k + 1, n, lo, hi, g);
                if (lo == k && hi == k + 1) return k + 1;
            }
            return k;
        }
        // last leaf of an odd count: right leaf child of [k - 2^tz(k), k]
        int h = topo_ctz((uint32_t)k);
        return k - (1 << h);
    }
    // odd k: right half of [k-1, k]
    if (k <= n - 2) {
        int32_t lo, hi, g;
        topo_range(k, n, lo, hi, g);
        if (lo == k - 1 && hi == k) return k;
    }
    return k - 1;
}

// Record fields of the node covering the block [lo, hi] = [j*2^L, ...] at
// level L (both halves non-empty): its index, split, parent and leaf flag.
struct TopoBlock { int32_t idx, gamma, parent, leaf; };
__host__ __device__ __forceinline__ TopoBlock topo_block(int32_t lo, int32_t hi, int level, int32_t n) {
    int32_t a_lo, a_hi, a_g;
    topo_range(lo, n, a_lo, a_hi, a_g);
    TopoBlock r;
    r.idx = (a_lo == lo && a_hi == hi) ? lo : hi;
    r.gamma = lo + (1 << (level - 1)) - 1;
    r.leaf = (level == 1 || hi == r.gamma + 1) ? 2 : 0;
    r.parent = topo_parent_internal(r.idx, lo, hi, n);
    return r;
}

// The same fields in a few integer operations for a block away from the
// right edge and the root: the block is complete, its sibling exists (so it
// is its parent's left child, numbered by its end, or right child, numbered
// by its start), and its parent's sibling exists (so the parent is numbered
// the same way one level up).  Other blocks take topo_block.
__host__ __device__ __forceinline__ TopoBlock topo_block_fast(int32_t lo, int32_t hi, int level, int32_t n) {
    const int32_t j = lo >> level, jp = j >> 1;
    const bool fast = ((int64_t)(j + 1) << level) <= n && ((int64_t)(j ^ 1) << level) < n &&
                      ((int64_t)(jp ^ 1) << (level + 1)) < n;
    if (!fast) return topo_block(lo, hi, level, n);
    TopoBlock r;
    r.idx = (j & 1) ? lo : hi;
    r.gamma = lo + (1 << (level - 1)) - 1;
    r.leaf = level == 1 ? 2 : 0;
    const int32_t plo = jp << (level + 1);
    r.parent = (jp & 1) ? plo : plo + (2 << level) - 1;
    return r;
}

// topo_parent_leaf in a few integer operations: the 2-leaf block [2j, 2j+1]
// (j = k / 2) is numbered by its end when it is a left child and by its
// start when a right child, whenever the block and its sibling exist.
__host__ __device__ __forceinline__ int32_t topo_parent_leaf_fast(int32_t k, int32_t n) {
    const int32_t j = k >> 1;
    if (2 * (int64_t)(j + 1) <= n && 2 * (int64_t)(j ^ 1) < n) return (j & 1) ? 2 * j : 2 * j + 1;
    return topo_parent_leaf(k, n);
}

}  // namespace ptgpu
