// host.h -- host-side pieces of the library: KD-tree build, scene loader,
// camera, seeds.  Plain C++17, no CUDA.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ptgpu.h"

namespace ptgpu {

// ---- KD tree (KDTree.cpp) ----------------------------------------------------
// Pointer tree held in arrays; node 0 is the root.  Leaves own the range
// [kmin, kmax) of `kn`, which lists shape ids in the reference's order (leaves
// in breadth-first order, each leaf's shapes in its vector order).
struct KdTree {
    std::vector<int32_t> leaf, left, right, depth, kmin, kmax;
    std::vector<ptgpu_bound> box;
    std::vector<int32_t> kn;
    int32_t max_depth = 0;
    int32_t szbuf = 0;
    int32_t node_count() const { return (int32_t)leaf.size(); }
};

int kd_build(const ptgpu_shape *shapes, uint32_t n, KdTree &out);
// KDTree::getTrees heap layout.  Returns PTGPU_E_RANGE if an index does not fit
// the int16 fields (the arrays are still filled, truncated like the reference).
int kd_heap_size(const KdTree &kd, int64_t *kng_cnt);
int kd_export_heap(const KdTree &kd, ptgpu_kd_node *kng, int64_t kng_cnt, int32_t *kn);
// The tree breadth-first with 32-bit fields (nodes must hold node_count()).
void kd_export_wide(const KdTree &kd, ptgpu_kd_node_wide *nodes);
// Traversal layout: 16 floats per internal node (see device.cuh), internal
// nodes numbered breadth-first; a root leaf is returned through root_first /
// root_count with no internal nodes.
void kd_trace_nodes(const KdTree &kd, std::vector<float> &nodes, int32_t *root_first,
                    int32_t *root_count, float root_box[6]);

// ---- scene loader (displayfunc.cpp) ---------------------------------------------
struct LoadedScene {
    std::vector<ptgpu_shape> shapes;
    uint32_t light_cnt = 0;
    ptgpu_camera camera{};
    bool walllight = true;
};
int read_scene(const char *path, int width, int height, LoadedScene &out, std::string &err);
void add_wall_light(LoadedScene &sc);      // AddWallLight (smallptGPU.cpp:1448-1459)

// OBJ model as read: x,y,z per vertex, 3 vertex indices per triangle (faces
// with more than three vertices fanned).  threads <= 0: one host thread per
// MiB of file, at most 16.
struct Obj {
    std::vector<float> v;
    std::vector<int32_t> tri;
};
bool read_obj(const char *path, Obj &obj, std::string &err, int threads = 0);

// The same scene without its model triangles expanded: segments in file
// order, each either shapes as read_scene gives them or one model kept as
// vertices + triangle indices with its placement and material.  Expanding
// every segment in order gives read_scene's shapes.
struct SceneSegment {
    bool model = false;
    std::vector<ptgpu_shape> shapes;             // !model
    Obj obj;                                     // model
    ptgpu_vec pos{}, scale{}, e{}, c{};
    int32_t refl = 0;
    int64_t count() const { return model ? (int64_t)(obj.tri.size() / 3) : (int64_t)shapes.size(); }
};
struct CompactScene {
    std::vector<SceneSegment> segs;
    uint32_t light_cnt = 0;
    ptgpu_camera camera{};
    bool walllight = true;
    int64_t count() const {
        int64_t n = 0;
        for (const SceneSegment &g : segs) n += g.count();
        return n;
    }
};
int read_scene_compact(const char *path, int width, int height, CompactScene &out, std::string &err);
void add_wall_light(CompactScene &sc);
// a model triangle as read_scene expands it (scaled, translated, area)
ptgpu_shape model_shape(const SceneSegment &g, size_t t);

// ---- camera / seeds -------------------------------------------------------------
void update_camera(ptgpu_camera *cam);     // UpdateCamera (displayfunc.cpp:732-756)
void make_seeds(uint64_t master, uint32_t *seeds, uint32_t count);

}  // namespace ptgpu
