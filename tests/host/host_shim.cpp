// host_shim.cpp -- test-only C entry points over the library's host code
// (KD-tree build, scene loader, camera, closed-form LBVH topology, the
// server's slot allocator and step policy), compiled
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
#include "../../ptgpu_pc_gb300/csrc/range_alloc.h"
#include "../../ptgpu_pc_gb300/csrc/step_policy.h"

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

int shim_kd_node_count() { return g_kd.node_count(); }

void shim_kd_export_wide(ptgpu_kd_node_wide *nodes, int32_t *kn) {
    ptgpu::kd_export_wide(g_kd, nodes);
    for (size_t i = 0; i < g_kd.kn.size(); ++i) kn[i] = g_kd.kn[i];
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

// read_obj with a given number of host threads; returns 1 on success and
// the counts, or 0 with the error text
static ptgpu::Obj g_obj;
int shim_read_obj(const char *path, int threads, int64_t *nv, int64_t *ntri, char *err, int errlen) {
    std::string e;
    g_obj = ptgpu::Obj();
    const bool ok = ptgpu::read_obj(path, g_obj, e, threads);
    *nv = (int64_t)(g_obj.v.size() / 3);
    *ntri = (int64_t)(g_obj.tri.size() / 3);
    std::strncpy(err, e.c_str(), errlen - 1);
    err[errlen - 1] = 0;
    return ok ? 1 : 0;
}
void shim_obj_get(float *v, int32_t *tri) {
    std::memcpy(v, g_obj.v.data(), g_obj.v.size() * sizeof(float));
    std::memcpy(tri, g_obj.tri.data(), g_obj.tri.size() * sizeof(int32_t));
}

// read_scene_compact (+ wall light), its segments expanded in order
static std::vector<ptgpu_shape> g_compact;
int shim_read_scene_compact(const char *path, int w, int h, int *n, int *light_cnt, int *segs) {
    ptgpu::CompactScene sc;
    std::string e;
    int st = ptgpu::read_scene_compact(path, w, h, sc, e);
    if (st != PTGPU_OK) return st;
    if (sc.walllight) ptgpu::add_wall_light(sc);
    g_compact.clear();
    for (const ptgpu::SceneSegment &g : sc.segs) {
        if (!g.model) g_compact.insert(g_compact.end(), g.shapes.begin(), g.shapes.end());
        else for (int64_t t = 0; t < g.count(); ++t) g_compact.push_back(ptgpu::model_shape(g, (size_t)t));
    }
    *n = (int)g_compact.size();
    *light_cnt = (int)sc.light_cnt;
    *segs = (int)sc.segs.size();
    return PTGPU_OK;
}
void shim_compact_get(ptgpu_shape *out) {
    std::memcpy(out, g_compact.data(), g_compact.size() * sizeof(ptgpu_shape));
}

void shim_update_camera(ptgpu_camera *cam) { ptgpu::update_camera(cam); }

void shim_make_seeds(uint64_t m, uint32_t *s, uint32_t n) { ptgpu::make_seeds(m, s, n); }

// the server's first-fit slot allocator
void *shim_ra_new() { return new ptgpu::RangeAlloc(); }
void shim_ra_delete(void *a) { delete static_cast<ptgpu::RangeAlloc *>(a); }
void shim_ra_grow(void *a, int64_t cap) { static_cast<ptgpu::RangeAlloc *>(a)->grow(cap); }
int shim_ra_alloc(void *a, int64_t n, int64_t *start) {
    return static_cast<ptgpu::RangeAlloc *>(a)->alloc(n, start) ? 1 : 0;
}
void shim_ra_release(void *a, int64_t start, int64_t n) { static_cast<ptgpu::RangeAlloc *>(a)->release(start, n); }
int64_t shim_ra_used(void *a) { return static_cast<ptgpu::RangeAlloc *>(a)->used; }
int64_t shim_ra_free_tail(void *a) { return static_cast<ptgpu::RangeAlloc *>(a)->free_tail(); }
// the free ranges in address order as (start, length) pairs; returns their count
int shim_ra_free(void *a, int64_t *out, int max_pairs) {
    int k = 0;
    for (const auto &r : static_cast<ptgpu::RangeAlloc *>(a)->free_) {
        if (k < max_pairs) { out[2 * k] = r.first; out[2 * k + 1] = r.second; }
        ++k;
    }
    return k;
}

// the serving step's request selection: indices into px (oldest first) into
// out; returns their count
int shim_step_selection(const int64_t *px, int n, int fill_cap, int64_t fill_px, int *out) {
    const std::vector<int> sel = ptgpu::step_selection(std::vector<int64_t>(px, px + n), fill_cap != 0, fill_px);
    for (size_t i = 0; i < sel.size(); ++i) out[i] = sel[i];
    return (int)sel.size();
}

}
