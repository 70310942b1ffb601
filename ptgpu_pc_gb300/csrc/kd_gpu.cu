// kd_gpu.cu -- the KD-tree build of KDTree::build (KDTree.cpp:89-182) on the
// GPU, with the reference's topology and float results.
//
// The tree is built one level at a time.  At a level every node owns a
// contiguous run of shape ids in the reference's vector order.  One CTA per
// node (k_kd_fold) stages its shapes' bounds and scaled midpoints in shared
// memory chunk by chunk, and one thread folds them in vector order exactly as
// the reference loop does: the box starts at shape 0's bound and grows by
// strict comparisons, the mean midpoint sums m * (1/n) over shapes 1..n-1 in
// order (float additions do not reassociate, so this sum is sequential), the
// axis is the longest extent.  The CTA then counts the shapes whose midpoint
// is <= the mean (they go right).  A node with one shape, or whose split
// leaves a side empty, is a leaf.  Exclusive scans over the level's nodes
// place the children of the internal nodes (in node order: the breadth-first
// numbering), their shapes in the next level's run, and the leaves' shapes in
// kn (leaves in breadth-first order, as KDTree::traverseTree lists them).
// k_kd_scatter then writes each internal node's shapes to its children, left
// ones first, each side in vector order (a stable partition: ranks come from
// one exclusive scan of the level's right flags).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "device.cuh"
#include "devbuf.h"
#include "host.h"
#include "lbvh.h"

namespace ptgpu {

namespace {

constexpr int kKdThreads = 256;
constexpr int kKdChunk = 1024;            // shapes staged per fold step

__device__ __forceinline__ void kd_shape(const float *__restrict__ verts, const uint8_t *__restrict__ type,
                                         int s, float b[6], float m[3]) {
    const float *v = verts + 9 * (size_t)s;
    if (type[s] == PTGPU_TRIANGLE) {        // KDTree.cpp:22-34, midpoint p3 / 3 (KDTree.cpp:55-57)
        const float x1 = v[0], y1 = v[1], z1 = v[2], x2 = v[3], y2 = v[4], z2 = v[5];
        const float x3 = v[6], y3 = v[7], z3 = v[8];
        b[0] = min2f(min2f(x1, x2), x3); b[1] = max2f(max2f(x1, x2), x3);
        b[2] = min2f(min2f(y1, y2), y3); b[3] = max2f(max2f(y1, y2), y3);
        b[4] = min2f(min2f(z1, z2), z3); b[5] = max2f(max2f(z1, z2), z3);
        m[0] = x3 / 3.0f; m[1] = y3 / 3.0f; m[2] = z3 / 3.0f;
    } else {                                 // KDTree.cpp:8-20, midpoint = centre
        const float px = v[0], py = v[1], pz = v[2], r = v[3];
        b[0] = px - r; b[1] = px + r; b[2] = py - r; b[3] = py + r; b[4] = pz - r; b[5] = pz + r;
        m[0] = px; m[1] = py; m[2] = pz;
    }
}

// Running minimum / maximum with the reference loop's outcome: a later value
// replaces the current one only when strictly smaller (larger), so among
// equal values the earliest stays and NaN never replaces (KDTree.h:35-44).
struct MinAt { float v; int i; };
__device__ __forceinline__ void take_min(MinAt &a, float v, int i) {
    if (v < a.v || (v == a.v && i < a.i)) { a.v = v; a.i = i; }
}
__device__ __forceinline__ void take_max(MinAt &a, float v, int i) {
    if (v > a.v || (v == a.v && i < a.i)) { a.v = v; a.i = i; }
}

// Per node of the level: box, split axis and value, count of shapes going
// right, leaf decision.  The box is reduced across the CTA over shapes
// 1..n-1 (index-aware, so the result is the sequential one) and then merged
// with shape 0's bound.  The mean midpoint is three sequential float sums
// (one per axis, in vector order): lane 0 of warps 0, 1 and 2 each sums one
// axis of a staged chunk while warps 3-7 stage the next chunk into the other
// half of a double buffer, so the sums run back to back at the adds' latency.
// node_* are the level's node arrays; out_* are indexed by the node's
// breadth-first id.
constexpr int kKdStageWarps = kKdThreads / 32 - 3;
__global__ void __launch_bounds__(kKdThreads) k_kd_fold(
    const float *__restrict__ verts, const uint8_t *__restrict__ type, const int32_t *__restrict__ ids,
    const int32_t *__restrict__ node_start, const int32_t *__restrict__ node_cnt,
    const int32_t *__restrict__ node_gid, float *__restrict__ node_split, int32_t *__restrict__ node_axis,
    uint32_t *__restrict__ n_internal_elems, uint32_t *__restrict__ n_leaf_elems,
    uint32_t *__restrict__ n_children, int32_t *__restrict__ node_rc, float *__restrict__ out_box,
    int32_t *__restrict__ out_leaf) {
    __shared__ float sm[2][3][kKdChunk];     // scaled midpoints, double-buffered
    __shared__ MinAt s_box[kKdThreads / 32][6];
    __shared__ float s_split, s_box0[6], s_mid[3];
    __shared__ int s_axis;
    __shared__ uint32_t s_right[kKdThreads / 32];
    const int k = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int start = node_start[k], cnt = node_cnt[k];
    const float recp = (float)(1.0 / (double)cnt);
    MinAt bx[6];
    for (int a = 0; a < 6; ++a) { bx[a].v = (a & 1) ? -INFINITY : INFINITY; bx[a].i = 0x7fffffff; }
    float mid = 0.f;                          // warps 0-2, lane 0: axis w
    const int nchunks = (cnt + kKdChunk - 1) / kKdChunk;
    const int st = tid - 3 * 32;              // staging thread index (warps 3-7)
    auto stage = [&](int c) {
        const int base = c * kKdChunk, m = min(kKdChunk, cnt - base);
        float(*buf)[kKdChunk] = sm[c & 1];
        for (int j = st; j < m; j += kKdStageWarps * 32) {
            float b[6], md[3];
            kd_shape(verts, type, ids[start + base + j], b, md);
            const int gi = base + j;
            if (gi == 0) {
                for (int a = 0; a < 6; ++a) s_box0[a] = b[a];
            } else {
                take_min(bx[0], b[0], gi); take_max(bx[1], b[1], gi);
                take_min(bx[2], b[2], gi); take_max(bx[3], b[3], gi);
                take_min(bx[4], b[4], gi); take_max(bx[5], b[5], gi);
            }
            for (int a = 0; a < 3; ++a) buf[a][j] = md[a] * recp;
        }
    };
    if (st >= 0) stage(0);
    __syncthreads();
    for (int c = 0; c < nchunks; ++c) {
        if (st >= 0) {
            if (c + 1 < nchunks) stage(c + 1);
        } else if (lane == 0) {               // KDTree.cpp:127-135: shapes 1..n-1 in order
            const int base = c * kKdChunk, m = min(kKdChunk, cnt - base);
            const float *v = sm[c & 1][w];
            for (int j = base == 0 ? 1 : 0; j < m; ++j) mid += v[j];
        }
        __syncthreads();
    }
    if (w < 3 && lane == 0) s_mid[w] = mid;
    // the box over shapes 1..n-1, then merged into shape 0's bound
    for (int o = 16; o > 0; o >>= 1) {
        for (int a = 0; a < 6; ++a) {
            const float v = __shfl_xor_sync(0xffffffffu, bx[a].v, o);
            const int i = __shfl_xor_sync(0xffffffffu, bx[a].i, o);
            if (a & 1) take_max(bx[a], v, i); else take_min(bx[a], v, i);
        }
    }
    if (lane == 0)
        for (int a = 0; a < 6; ++a) s_box[w][a] = bx[a];
    __syncthreads();
    if (tid == 0) {
        float box[6];
        for (int a = 0; a < 6; ++a) {
            MinAt r = s_box[0][a];
            for (int q = 1; q < kKdThreads / 32; ++q) {
                if (a & 1) take_max(r, s_box[q][a].v, s_box[q][a].i);
                else take_min(r, s_box[q][a].v, s_box[q][a].i);
            }
            const float b0 = s_box0[a];
            const bool later = r.i != 0x7fffffff && ((a & 1) ? (r.v > b0) : (r.v < b0));
            box[a] = later ? r.v : b0;
        }
        const float xd = box[1] - box[0], yd = box[3] - box[2], zd = box[5] - box[4];
        const int axis = xd >= yd ? (xd >= zd ? 0 : 2) : (yd >= zd ? 1 : 2);   // KDTree.cpp:72-86
        s_axis = axis;
        s_split = s_mid[axis];
        float *ob = out_box + 6 * (size_t)node_gid[k];
        for (int a = 0; a < 6; ++a) ob[a] = box[a];
    }
    __syncthreads();
    // shapes going right: split >= midpoint (KDTree.cpp:142-155)
    const int axis = s_axis;
    const float split = s_split;
    uint32_t right = 0;
    for (int j = tid; j < cnt; j += kKdThreads) {
        float b[6], md[3];
        kd_shape(verts, type, ids[start + j], b, md);
        right += (split >= md[axis]) ? 1u : 0u;
    }
    for (int o = 16; o > 0; o >>= 1) right += __shfl_xor_sync(0xffffffffu, right, o);
    if (lane == 0) s_right[w] = right;
    __syncthreads();
    if (tid == 0) {
        uint32_t rc = 0;
        for (int q = 0; q < kKdThreads / 32; ++q) rc += s_right[q];
        const bool leaf = cnt <= 1 || rc == 0 || rc == (uint32_t)cnt;
        out_leaf[node_gid[k]] = leaf ? 1 : 0;
        node_split[k] = split;
        node_axis[k] = axis;
        node_rc[k] = (int32_t)rc;
        n_internal_elems[k] = leaf ? 0u : (uint32_t)cnt;
        n_leaf_elems[k] = leaf ? (uint32_t)cnt : 0u;
        n_children[k] = leaf ? 0u : 2u;
    }
}

// Per shape of the level: 1 when it goes right (internal nodes only).
__global__ void k_kd_flags(const float *__restrict__ verts, const uint8_t *__restrict__ type,
                           const int32_t *__restrict__ ids, const int32_t *__restrict__ enode, int E,
                           const int32_t *__restrict__ node_gid, const float *__restrict__ node_split,
                           const int32_t *__restrict__ node_axis, const int32_t *__restrict__ out_leaf,
                           uint32_t *__restrict__ flag) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int k = enode[e];
    uint32_t f = 0;
    if (!out_leaf[node_gid[k]]) {
        float b[6], md[3];
        kd_shape(verts, type, ids[e], b, md);
        f = (node_split[k] >= md[node_axis[k]]) ? 1u : 0u;
    }
    flag[e] = f;
}

// Per node: its children's entries for the next level, or its kn range.
__global__ void k_kd_nodes(int L, const int32_t *__restrict__ node_start, const int32_t *__restrict__ node_cnt,
                           const int32_t *__restrict__ node_gid, const int32_t *__restrict__ node_rc,
                           const uint32_t *__restrict__ elem_off, const uint32_t *__restrict__ kn_off,
                           const uint32_t *__restrict__ child_off, int next_gid_base, int kn_base, int depth,
                           int32_t *__restrict__ next_start, int32_t *__restrict__ next_cnt,
                           int32_t *__restrict__ next_gid, int32_t *__restrict__ out_left,
                           int32_t *__restrict__ out_right, int32_t *__restrict__ out_kmin,
                           int32_t *__restrict__ out_kmax, int32_t *__restrict__ out_depth,
                           const int32_t *__restrict__ out_leaf) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L) return;
    const int gid = node_gid[k], cnt = node_cnt[k];
    out_depth[gid] = depth;
    if (out_leaf[gid]) {
        const int kb = kn_base + (int)kn_off[k];
        out_kmin[gid] = kb;
        out_kmax[gid] = kb + cnt;
        out_left[gid] = -1;
        out_right[gid] = -1;
        return;
    }
    const int rc = node_rc[k], lc = cnt - rc, c0 = (int)child_off[k], base = (int)elem_off[k];
    out_left[gid] = next_gid_base + c0;
    out_right[gid] = next_gid_base + c0 + 1;
    out_kmin[gid] = 0;
    out_kmax[gid] = 0;
    next_start[c0] = base;
    next_cnt[c0] = lc;
    next_gid[c0] = next_gid_base + c0;
    next_start[c0 + 1] = base + lc;
    next_cnt[c0 + 1] = rc;
    next_gid[c0 + 1] = next_gid_base + c0 + 1;
}

// Per shape: its place in kn (leaf node) or in the next level, left shapes of
// a node first, each side in order (ranks from the global scan of the flags).
__global__ void k_kd_scatter(const int32_t *__restrict__ ids, const int32_t *__restrict__ enode, int E,
                             const int32_t *__restrict__ node_start, const int32_t *__restrict__ node_cnt,
                             const int32_t *__restrict__ node_gid, const int32_t *__restrict__ node_rc,
                             const uint32_t *__restrict__ elem_off, const uint32_t *__restrict__ kn_off,
                             const uint32_t *__restrict__ child_off, const uint32_t *__restrict__ scan,
                             int kn_base, const int32_t *__restrict__ out_leaf, int32_t *__restrict__ ids_next,
                             int32_t *__restrict__ enode_next, int32_t *__restrict__ kn) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int k = enode[e], start = node_start[k];
    if (out_leaf[node_gid[k]]) {
        kn[kn_base + (int)kn_off[k] + (e - start)] = ids[e];
        return;
    }
    const int lc = node_cnt[k] - node_rc[k];
    const uint32_t rbefore = scan[e] - scan[start];
    const bool right = scan[e + 1] != scan[e];
    const int pos = right ? (int)elem_off[k] + lc + (int)rbefore : (int)elem_off[k] + (e - start) - (int)rbefore;
    ids_next[pos] = ids[e];
    enode_next[pos] = (int)child_off[k] + (right ? 1 : 0);
}

// Exclusive scan of n words into out[0..n] (out[n] = total), 1024 per CTA.
__global__ void __launch_bounds__(1024) k_scan_block(const uint32_t *__restrict__ in, uint32_t *__restrict__ out,
                                                     int n, uint32_t *__restrict__ sums) {
    __shared__ uint32_t s_w[32];
    const int i = blockIdx.x * 1024 + threadIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t v = i < n ? in[i] : 0u;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_w[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = s_w[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        s_w[lane] = t;
    }
    __syncthreads();
    const uint32_t incl = x + (w ? s_w[w - 1] : 0u);
    if (i < n) out[i] = incl - v;
    if (threadIdx.x == 1023) sums[blockIdx.x] = incl;
}

__global__ void k_scan_add(uint32_t *__restrict__ out, int n, const uint32_t *__restrict__ offs) {
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += offs[blockIdx.x];
}

__global__ void k_scan_total(uint32_t *__restrict__ out, const uint32_t *__restrict__ in, int n) {
    out[n] = n > 0 ? out[n - 1] + in[n - 1] : 0u;
}

// tmp: room for the block sums of every recursion level (n / 512 + 64 words)
cudaError_t scan_exclusive(const uint32_t *in, uint32_t *out, int n, uint32_t *tmp, cudaStream_t s) {
    if (n <= 0) {
        return cudaMemsetAsync(out, 0, sizeof(uint32_t), s);
    }
    const int nb = (n + 1023) / 1024;
    k_scan_block<<<nb, 1024, 0, s>>>(in, out, n, tmp);
    if (nb > 1) {
        uint32_t *offs = tmp + nb;
        cudaError_t e = scan_exclusive(tmp, offs, nb, offs + nb + 1, s);
        if (e != cudaSuccess) return e;
        k_scan_add<<<nb, 1024, 0, s>>>(out, n, offs);
    }
    k_scan_total<<<1, 1, 0, s>>>(out, in, n);
    return cudaGetLastError();
}

}  // namespace

struct KdScratch {
    DevBuf ids_a, ids_b, en_a, en_b, flag, fscan, nodes_a, nodes_b, split, axis, rc, n_int, n_leaf, n_child;
    DevBuf elem_off, kn_off, child_off, scan_tmp, kn, leaf, left, right, kmin, kmax, depth, box;
};

KdScratch *kd_scratch_create() { return new KdScratch(); }
void kd_scratch_destroy(KdScratch *w) {
    if (!w) return;
    DevBuf *bs[] = {&w->ids_a, &w->ids_b, &w->en_a, &w->en_b, &w->flag, &w->fscan, &w->nodes_a, &w->nodes_b, &w->split, &w->axis, &w->rc,
                    &w->n_int, &w->n_leaf, &w->n_child, &w->elem_off, &w->kn_off, &w->child_off,
                    &w->scan_tmp, &w->kn, &w->leaf, &w->left, &w->right, &w->kmin, &w->kmax,
                    &w->depth, &w->box};
    for (DevBuf *b : bs) b->release();
    delete w;
}

#define KK(expr)                                            \
    do {                                                    \
        cudaError_t e_ = (expr);                            \
        if (e_ != cudaSuccess) return e_;                   \
    } while (0)

// The KD tree of n shapes (build vertices and types on the device), into kd
// with breadth-first node ids.
cudaError_t kd_build_gpu(const float *verts, const uint8_t *type, uint32_t n, KdTree &kd, KdScratch &w,
                         cudaStream_t s) {
    kd = KdTree();
    if (n == 0) return cudaSuccess;
    const size_t N = n, M = 2 * (size_t)n + 2;   // at most 2n - 1 nodes
    KK(w.ids_a.ensure(N * 4));
    KK(w.ids_b.ensure(N * 4));
    KK(w.en_a.ensure(N * 4));
    KK(w.en_b.ensure(N * 4));
    KK(w.flag.ensure(N * 4));
    KK(w.fscan.ensure((N + 1) * 4));
    KK(w.nodes_a.ensure(3 * N * 4));   // start, count, gid per level node (at most n per level)
    KK(w.nodes_b.ensure(3 * N * 4));
    KK(w.split.ensure(N * 4));
    KK(w.axis.ensure(N * 4));
    KK(w.rc.ensure(N * 4));
    KK(w.n_int.ensure(N * 4));
    KK(w.n_leaf.ensure(N * 4));
    KK(w.n_child.ensure(N * 4));
    KK(w.elem_off.ensure((N + 1) * 4));
    KK(w.kn_off.ensure((N + 1) * 4));
    KK(w.child_off.ensure((N + 1) * 4));
    KK(w.scan_tmp.ensure((N / 256 + 256) * 4));
    KK(w.kn.ensure(N * 4));
    KK(w.leaf.ensure(M * 4));
    KK(w.left.ensure(M * 4));
    KK(w.right.ensure(M * 4));
    KK(w.kmin.ensure(M * 4));
    KK(w.kmax.ensure(M * 4));
    KK(w.depth.ensure(M * 4));
    KK(w.box.ensure(M * 6 * 4));
    // level 0: the root holds shapes 0..n-1 in order
    std::vector<int32_t> ident(n);
    for (uint32_t i = 0; i < n; ++i) ident[i] = (int32_t)i;
    KK(cudaMemcpyAsync(w.ids_a.p, ident.data(), N * 4, cudaMemcpyHostToDevice, s));
    const int32_t root[3] = {0, (int32_t)n, 0};
    int32_t *lv = w.nodes_a.as<int32_t>(), *lv_next = w.nodes_b.as<int32_t>();
    KK(cudaMemcpyAsync(lv, &root[0], 4, cudaMemcpyHostToDevice, s));
    KK(cudaMemcpyAsync(lv + N, &root[1], 4, cudaMemcpyHostToDevice, s));
    KK(cudaMemcpyAsync(lv + 2 * N, &root[2], 4, cudaMemcpyHostToDevice, s));
    KK(cudaMemsetAsync(w.en_a.p, 0, N * 4, s));
    int32_t *ids = w.ids_a.as<int32_t>(), *ids_next = w.ids_b.as<int32_t>();
    int32_t *en = w.en_a.as<int32_t>(), *en_next = w.en_b.as<int32_t>();
    int L = 1, E = (int)n, gid_base = 0, kn_base = 0, depth = 0, total_nodes = 1;
    while (L > 0) {
        k_kd_fold<<<L, kKdThreads, 0, s>>>(verts, type, ids, lv, lv + N, lv + 2 * N, w.split.as<float>(),
                                          w.axis.as<int32_t>(), w.n_int.as<uint32_t>(), w.n_leaf.as<uint32_t>(),
                                          w.n_child.as<uint32_t>(), w.rc.as<int32_t>(), w.box.as<float>(),
                                          w.leaf.as<int32_t>());
        KK(cudaGetLastError());
        KK(scan_exclusive(w.n_int.as<uint32_t>(), w.elem_off.as<uint32_t>(), L, w.scan_tmp.as<uint32_t>(), s));
        KK(scan_exclusive(w.n_leaf.as<uint32_t>(), w.kn_off.as<uint32_t>(), L, w.scan_tmp.as<uint32_t>(), s));
        KK(scan_exclusive(w.n_child.as<uint32_t>(), w.child_off.as<uint32_t>(), L, w.scan_tmp.as<uint32_t>(), s));
        const int next_base = gid_base + L;
        k_kd_flags<<<(E + 255) / 256, 256, 0, s>>>(verts, type, ids, en, E, lv + 2 * N, w.split.as<float>(),
                                                  w.axis.as<int32_t>(), w.leaf.as<int32_t>(),
                                                  w.flag.as<uint32_t>());
        KK(cudaGetLastError());
        KK(scan_exclusive(w.flag.as<uint32_t>(), w.fscan.as<uint32_t>(), E, w.scan_tmp.as<uint32_t>(), s));
        k_kd_nodes<<<(L + 255) / 256, 256, 0, s>>>(
            L, lv, lv + N, lv + 2 * N, w.rc.as<int32_t>(), w.elem_off.as<uint32_t>(), w.kn_off.as<uint32_t>(),
            w.child_off.as<uint32_t>(), next_base, kn_base, depth, lv_next, lv_next + N, lv_next + 2 * N,
            w.left.as<int32_t>(), w.right.as<int32_t>(), w.kmin.as<int32_t>(), w.kmax.as<int32_t>(),
            w.depth.as<int32_t>(), w.leaf.as<int32_t>());
        KK(cudaGetLastError());
        k_kd_scatter<<<(E + 255) / 256, 256, 0, s>>>(
            ids, en, E, lv, lv + N, lv + 2 * N, w.rc.as<int32_t>(), w.elem_off.as<uint32_t>(),
            w.kn_off.as<uint32_t>(), w.child_off.as<uint32_t>(), w.fscan.as<uint32_t>(), kn_base,
            w.leaf.as<int32_t>(), ids_next, en_next, w.kn.as<int32_t>());
        KK(cudaGetLastError());
        uint32_t tot[3] = {0, 0, 0};
        KK(cudaMemcpyAsync(&tot[0], w.child_off.as<uint32_t>() + L, 4, cudaMemcpyDeviceToHost, s));
        KK(cudaMemcpyAsync(&tot[1], w.kn_off.as<uint32_t>() + L, 4, cudaMemcpyDeviceToHost, s));
        KK(cudaMemcpyAsync(&tot[2], w.elem_off.as<uint32_t>() + L, 4, cudaMemcpyDeviceToHost, s));
        KK(cudaStreamSynchronize(s));
        E = (int)tot[2];
        kd.max_depth = depth;
        kn_base += (int)tot[1];
        gid_base = next_base;
        L = (int)tot[0];
        total_nodes += L;
        ++depth;
        std::swap(ids, ids_next);
        std::swap(en, en_next);
        std::swap(lv, lv_next);
    }
    // the tree into host arrays (breadth-first ids)
    const size_t T = (size_t)total_nodes;
    kd.leaf.resize(T); kd.left.resize(T); kd.right.resize(T); kd.depth.resize(T);
    kd.kmin.resize(T); kd.kmax.resize(T); kd.box.resize(T); kd.kn.resize(n);
    KK(cudaMemcpyAsync(kd.leaf.data(), w.leaf.p, T * 4, cudaMemcpyDeviceToHost, s));
    KK(cudaMemcpyAsync(kd.left.data(), w.left.p, T * 4, cudaMemcpyDeviceToHost, s));
    KK(cudaMemcpyAsync(kd.right.data(), w.right.p, T * 4, cudaMemcpyDeviceToHost, s));
    KK(cudaMemcpyAsync(kd.depth.data(), w.depth.p, T * 4, cudaMemcpyDeviceToHost, s));
    KK(cudaMemcpyAsync(kd.kmin.data(), w.kmin.p, T * 4, cudaMemcpyDeviceToHost, s));
    KK(cudaMemcpyAsync(kd.kmax.data(), w.kmax.p, T * 4, cudaMemcpyDeviceToHost, s));
    KK(cudaMemcpyAsync(kd.box.data(), w.box.p, T * sizeof(ptgpu_bound), cudaMemcpyDeviceToHost, s));
    KK(cudaMemcpyAsync(kd.kn.data(), w.kn.p, N * 4, cudaMemcpyDeviceToHost, s));
    KK(cudaStreamSynchronize(s));
    kd.szbuf = (int32_t)n;
    return cudaSuccess;
}

}  // namespace ptgpu
