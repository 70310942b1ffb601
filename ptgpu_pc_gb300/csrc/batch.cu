// batch.cu -- device helpers of the batched renderer (batch.cpp).
#include <cstdint>
#include <cuda_runtime.h>

#include "lbvh.h"

namespace ptgpu {

// rec.root holds the global index of the scene's root node; its bound is the
// traversal's root box
__global__ void k_fill_roots(BatchScene *recs, int n, const ptgpu_bvh_node *__restrict__ btn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ptgpu_bound b = btn[recs[i].root].bound;
    float *r = recs[i].root_box;
    r[0] = b.min_x; r[1] = b.max_x; r[2] = b.min_y; r[3] = b.max_y; r[4] = b.min_z; r[5] = b.max_z;
}

// Each leaf climbs its tree through nParent to the root (local node 0) and
// counts the internal nodes on the way; the walk is capped at 4096 steps.
__global__ void k_tree_depth(const ptgpu_bvh_node *__restrict__ btn,
                             const ptgpu_bvh_node *__restrict__ btl,
                             const int32_t *__restrict__ seg_off, int n_segs, int n, int *depth) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int d = 0;
    if (i < n) {
        int lo = 0, hi = n_segs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (seg_off[mid] <= i) lo = mid; else hi = mid - 1;
        }
        const int off = seg_off[lo], ns = seg_off[lo + 1] - off;
        const ptgpu_bvh_node *tn = btn + (off - lo);
        int p = btl[i].nParent;
        while (p >= 0 && p < ns - 1 && d < 4096) {
            ++d;
            if (p == 0) break;
            p = tn[p].nParent;
        }
    }
    for (int o = 16; o > 0; o >>= 1) d = max(d, __shfl_xor_sync(0xffffffffu, d, o));
    if ((threadIdx.x & 31) == 0 && d > 0) atomicMax(depth, d);
}

cudaError_t launch_fill_roots(BatchScene *recs, int n, const ptgpu_bvh_node *btn, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_fill_roots<<<(n + 127) / 128, 128, 0, s>>>(recs, n, btn);
    return cudaGetLastError();
}

cudaError_t launch_tree_depth(const ptgpu_bvh_node *btn, const ptgpu_bvh_node *btl,
                              const int32_t *seg_off, int n_segs, int n_total, int *depth,
                              cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(depth, 0, sizeof(int), s);
    if (e != cudaSuccess || n_total <= 0) return e;
    k_tree_depth<<<(n_total + 255) / 256, 256, 0, s>>>(btn, btl, seg_off, n_segs, n_total, depth);
    return cudaGetLastError();
}

}  // namespace ptgpu
