// host_shim.cpp -- test-only C entry points over the library's host code
// (KD-tree build, scene loader, camera, closed-form LBVH topology), compiled
// without CUDA by the CPU tests.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#define __host__
#define __device__
#define __forceinline__ inline
#include "../../ptgpu_pc_gb300/csrc/lbvh_topo.cuh"
#include "../../ptgpu_pc_gb300/csrc/host.h"

extern "C" {

// min, max, gamma, parent, leaf flag for every internal node; leaf parents
void shim_topology(int n, int *mn, int *mx, int *gamma, int *parent, int *leaf, int *leaf_parent) {
    for (int i = 0; i + 1 < n; ++i) {
        ptgpu::TopoNode t = ptgpu::topo_node(i, n);
        mn[i] = t.lo; mx[i] = t.hi; gamma[i] = t.gamma; parent[i] = t.parent;
        leaf[i] = (t.left_leaf || t.right_leaf) ? 2 : 0;
    }
    for (int k = 0; k < n; ++k) leaf_parent[k] = ptgpu::topo_parent_leaf(k, n);
}

// Every block of 2^L leaves with both halves non-empty: the short form of its
// record fields against the general one, and the general one against the
// node that carries its index; every leaf's parent in short and general
// form.  Returns the number of mismatches.
int shim_check_blocks(int n) {
    int bad = 0;
    for (int level = 1; level < 31 && (1 << (level - 1)) < n; ++level) {
        for (int64_t lo = 0; lo < n; lo += (int64_t)1 << level) {
            if (lo + ((int64_t)1 << (level - 1)) >= n) continue;          // right half empty
            const int hi = (int)std::min<int64_t>(lo + ((int64_t)1 << level), n) - 1;
            const ptgpu::TopoBlock g = ptgpu::topo_block((int)lo, hi, level, n);
            const ptgpu::TopoBlock f = ptgpu::topo_block_fast((int)lo, hi, level, n);
            if (g.idx != f.idx || g.gamma != f.gamma || g.parent != f.parent || g.leaf != f.leaf) ++bad;
            const ptgpu::TopoNode t = ptgpu::topo_node(g.idx, n);
            const int leaf = (t.left_leaf || t.right_leaf) ? 2 : 0;
            if (t.lo != (int)lo || t.hi != hi || t.gamma != g.gamma || t.parent != g.parent || leaf != g.leaf) ++bad;
        }
    }
    for (int k = 0; k < n; ++k)
        if (ptgpu::topo_parent_leaf_fast(k, n) != ptgpu::topo_parent_leaf(k, n)) ++bad;
    return bad;
}

static ptgpu::KdTree g_kd;

int shim_kd_build(const ptgpu_shape *shapes, int n, int *max_depth, int *szbuf, int64_t *heap) {
    int st = ptgpu::kd_build(shapes, (uint32_t)n, g_kd);
    *max_depth = g_kd.max_depth;
    *szbuf = g_kd.szbuf;
    int r = ptgpu::kd_heap_size(g_kd, heap);
    (void)r;
    return st;
}

int shim_kd_export(ptgpu_kd_node *kng, int64_t cnt, int32_t *kn) {
    return ptgpu::kd_export_heap(g_kd, kng, cnt, kn);
}

static ptgpu::LoadedScene g_scene;

int shim_read_scene(const char *path, int w, int h, int *n, int *light_cnt, int *walllight,
                    char *err, int errlen) {
    std::string e;
    int st = ptgpu::read_scene(path, w, h, g_scene, e);
    if (st == PTGPU_OK && g_scene.walllight) ptgpu::add_wall_light(g_scene);
    *n = (int)g_scene.shapes.size();
    *light_cnt = (int)g_scene.light_cnt;
    *walllight = g_scene.walllight ? 1 : 0;
    std::strncpy(err, e.c_str(), errlen - 1);
    err[errlen - 1] = 0;
    return st;
}

void shim_scene_get(ptgpu_shape *out, ptgpu_camera *cam) {
    std::memcpy(out, g_scene.shapes.data(), g_scene.shapes.size() * sizeof(ptgpu_shape));
    *cam = g_scene.camera;
}

void shim_update_camera(ptgpu_camera *cam) { ptgpu::update_camera(cam); }

void shim_make_seeds(uint64_t m, uint32_t *s, uint32_t n) { ptgpu::make_seeds(m, s, n); }

}
