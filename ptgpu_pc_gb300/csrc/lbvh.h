// lbvh.h -- host-side interface of the GPU LBVH build and of the traversal
// data preparation (lbvh.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/ptgpu.h"
#include "types.h"

namespace ptgpu {

// Per-build device state, zeroed by the first kernel of every build.
struct BuildState {
    uint32_t hist[5][256];      // digit histograms of the radix passes (the fifth:
                                // the segment pass of a batched build)
    uint32_t tile_counter[5];   // dynamic tile ids of the onesweep passes
    uint32_t cmin[3], cmax[3];  // centroid bounds as order-preserving uints
    uint32_t error;             // bit 0: a look-back wait gave up
    uint32_t top_ticket;
    uint32_t wait_limit;        // polls a look-back may wait before it gives up
};

// Polls (about 32 ns apart) a radix-sort look-back waits for a predecessor
// tile before the build gives up with PTGPU_E_TIMEOUT.
constexpr uint32_t kDefaultWaitLimit = 1u << 22;

struct LbvhBuffers {
    const float *verts;         // 9 floats per shape (p1,p2,p3 or centre,rad)
    const uint8_t *type;        // PTGPU_SPHERE / PTGPU_TRIANGLE per shape
    float4 *aabbs;              // 2 per shape: (min_x,max_x,min_y,max_y), (min_z,max_z,-,-)
    float4 *leaf_bounds;        // the same records in sorted (leaf) order (batched build)
    uint32_t *keys;             // ~Morton code per shape (sort key)
    uint32_t *keys_alt, *keys_tmp;
    int32_t *vals_alt, *vals_tmp;
    int32_t *sorted;            // sorted_geometry_indices
    uint32_t *status;           // look-back words, sort_status_words(n)
    BuildState *state;
    float *block_bounds;        // 6 floats per block at the tile level and above
    uint32_t *arrivals;         // arrival counters of the blocks above the tiles
    ptgpu_bvh_node *btn, *btl;  // the reference's output arrays
    uint32_t wait_limit = kDefaultWaitLimit;   // BuildState::wait_limit of the build
};

size_t sort_status_words(int n);   // look-back words of all (five) passes
size_t block_bound_count(int n);   // blocks at the tile level and above (+ slack)

cudaError_t launch_unpack_shapes(const ptgpu_shape *d_shapes, int n, float *verts, uint8_t *type,
                                 float4 *prims, Material *mats, cudaStream_t s);
cudaError_t launch_lbvh_build(const LbvhBuffers &b, int n, int all_tri, int sm_count,
                              cudaStream_t s);
// Segmented build: one LBVH per segment (scene) of the concatenated shape
// arrays, all in one pass of each kernel.  btn holds the segments' internal
// nodes back to back (segment s from seg_off[s] - s), btl their leaves (from
// seg_off[s]), block_bounds / arrivals their per-level blocks (from bb_off[s]).
// Every segment has at least two shapes.
constexpr int kMaxSegments = 256;
struct SegState { uint32_t cmin[3], cmax[3]; };
struct SegBuild {
    const int32_t *seg_off;     // n_segs + 1 shape offsets
    const int32_t *tile_off;    // n_segs + 1 offsets of the segments' emission tiles
    const int32_t *bb_off;      // n_segs + 1 offsets into block_bounds / arrivals
    SegState *seg_state;        // n_segs
    int32_t n_segs;
    int32_t n_tiles;            // tile_off[n_segs]
    int64_t n_blocks;           // bb_off[n_segs]
};
size_t seg_block_bound_count(int n);   // block_bound_count of one segment
int emission_tiles(int n);             // emission tiles of one segment
cudaError_t launch_lbvh_build_seg(const LbvhBuffers &b, int n_total, const SegBuild &sb,
                                  int sm_count, cudaStream_t s);
cudaError_t launch_treelet(ptgpu_bvh_node *btn, ptgpu_bvh_node *btl, int n, int *counters,
                           float *cost, int sweeps, cudaStream_t s);
// The same rounds for every segment of a batched build in one launch each
// (segment g: leaves at btl + seg_off[g], internal nodes / counters / costs
// at seg_off[g] - g); counters and cost hold n_total - n_segs entries.
cudaError_t launch_treelet_seg(ptgpu_bvh_node *btn, ptgpu_bvh_node *btl, const int32_t *seg_off, int n_segs,
                               int n_total, int *counters, float *cost, int sweeps, cudaStream_t s);
// node_base / shape_base: added to the child references and shape ids
// written (a segment's place in the shared arrays of a batch; 0 otherwise)
cudaError_t launch_abi_to_trace(const ptgpu_bvh_node *btn, const ptgpu_bvh_node *btl, int n,
                                const float4 *prims0, float4 *nodes, float4 *prims,
                                int32_t *prim_id, cudaStream_t s, int node_base = 0,
                                int shape_base = 0);
cudaError_t launch_collapse4(const float4 *nodes2, int n_int, float4 *nodes4, cudaStream_t s);
cudaError_t launch_gather_prims(const int32_t *order, int count, const float4 *prims0,
                                float4 *prims, cudaStream_t s);
// shapes with a BVH build's index / morton_code / b written into out
cudaError_t launch_export_shapes(const ptgpu_shape *shapes, ptgpu_shape *out, const float *verts,
                                 const uint8_t *type, const uint32_t *keys, int n, cudaStream_t s);

// trace.cu
// One scene of a batched render.  Node, primitive, material and light
// indices are global: the scenes' arrays are concatenated.
struct BatchScene {
    ptgpu_camera cam;
    int32_t width, height, passes, max_depth;
    int32_t start_sample;
    int32_t root;               // global node index of the scene's root (>= 2 shapes)
    int32_t n_shapes;
    int32_t skip;               // global id of the scene's last shape
    int32_t shape0;             // global id of the scene's first shape
    int32_t light_first, n_lights;
    int32_t pad;
    int64_t pix_off;            // first pixel in colors/pixels; seeds at 2 * pix_off
    float root_box[6];
};

struct RenderArgs {
    TraceView tv;
    const Material *mats;
    const float4 *prims0;       // shape-order prims (geometry of shape 0 for a
                                // hit reported beyond t = 1e20)
    const LightRec *lights;
    int32_t n_lights;
    ptgpu_camera cam;
    int32_t width, height;
    int32_t start_sample, passes;
    int32_t max_depth;
    int32_t rtl;                // evaluate light-sample random pairs right-to-left
    int32_t rr_depth;           // > 0: throughput Russian roulette from that hit depth on
    ptgpu_vec *colors;          // W*H, row-flipped (RadianceGPU)
    uint32_t *pixels;           // W*H RGBA8
    uint32_t *seeds;            // 2*W*H
    unsigned long long *stats;  // optional traversal counters (6 words)
    unsigned int *pixel_counter;// next pixel to hand out (zeroed per launch)
    // single-scene renders: the hand-out order (a permutation of the pixels;
    // null: row order) and each pixel's measured work, written as it finishes
    // (null: not measured).  Which lane renders a pixel when does not change
    // its result, so the order only decides how the frame's tail packs.
    const int32_t *order;
    uint32_t *cost;
    int32_t max_ctas;           // grid cap (resident CTAs); 0 = one lane per pixel
    int32_t refill;             // 32nds of a warp's live lanes that wait before it
                                // shades (0: the default)
    // batched render (scenes != null): the scene records in hand-out order,
    // their first pixel in that order (n_scenes + 1 entries); the single-scene
    // fields above (camera, size, passes, lights, depth, root) are unused
    const BatchScene *scenes;
    const int64_t *pix_start;
    int32_t n_scenes;
};
cudaError_t launch_render(const RenderArgs &a, int block, cudaStream_t s);
// Image encoding (image.cu).  PPM "P3" text of the RGBA8 pixels: row_off
// (h + 1 words) gets each output row's character offset and the total in
// row_off[h]; the text (without the header) is then written to out.
cudaError_t launch_ppm_length(const uint32_t *pixels, int w, int h, uint64_t *row_off, cudaStream_t s);
cudaError_t launch_ppm_write(const uint32_t *pixels, int w, int h, const uint64_t *row_off, char *out,
                             cudaStream_t s);
// PFM float RGB of the row-flipped colour buffer, bottom row first (3*w*h floats)
cudaError_t launch_pfm(const ptgpu_vec *colors, int w, int h, float *out, int sm_count, cudaStream_t s);
// The next frame's hand-out order from this frame's per-pixel work: pixels in
// decreasing work (logarithmic classes, 8 per power of two; any order inside
// a class), so the longest pixel chains start first and the frame ends on
// short ones.  scratch: 2 * kOrderScratchWords words.
constexpr int kOrderScratchWords = 1024;
cudaError_t launch_pixel_order(const uint32_t *cost, int32_t *order, uint32_t *scratch, int npx, cudaStream_t s);
// A batched render (binary nodes; stack 32, 64 or 128 entries) on `grid` resident
// CTAs from render_batch_grid; the launch only enqueues stream work (the
// pixel counter's reset and the kernel), so it can be captured in a graph.
int render_stack_for_depth(int depth);   // 32, 64 or 128 entries for a tree depth
int render_batch_grid(int block, int stack, int max_ctas);
cudaError_t launch_render_batch(const RenderArgs &a, int block, int stack, int grid, cudaStream_t s);
// batch.cu: each segment's root bound into its scene record; the deepest
// leaf of every segment's tree (internal nodes on its path) into *depth
cudaError_t launch_fill_roots(BatchScene *recs, int n, const ptgpu_bvh_node *btn, cudaStream_t s);
cudaError_t launch_tree_depth(const ptgpu_bvh_node *btn, const ptgpu_bvh_node *btl,
                              const int32_t *seg_off, int n_segs, int n_total, int *depth,
                              cudaStream_t s);

// wavefront.cu: path state for `paths` slots (struct of arrays, carved from
// one allocation of wf_carve_bytes) and the queues between the kernels
struct WfArgs {
    RenderArgs r;
    int32_t paths;
    float4 *o, *d, *rad, *tp, *col;
    uint2 *seeds;
    int4 *meta;                 // (depth, specularBounce, passes done, pixel)
    int2 *nee;                  // (first shadow entry, count)
    float2 *hit;                // (t, prim as int bits; -2 = miss)
    int *ext_in, *ext_out, *pend;
    float4 *sh_o, *sh_d, *sh_c; // shadow ray origin+maxt, dir+path, contribution
    unsigned char *sh_vis;
    unsigned *counters;         // ext in, ext out, shadow, pending
};
constexpr int kWfMaxLights = 8;
size_t wf_carve_bytes(int paths, int n_lights);
void wf_carve(WfArgs &a, void *base, int paths, int n_lights);
cudaError_t launch_wavefront(WfArgs a, int iterations, int grid, cudaStream_t s);
// counter: a device word for the persistent kernel (null: one thread per ray)
// stats (with counter): node visits and primitive tests added to stats[0..1]
cudaError_t launch_trace_closest(const TraceView &tv, const ptgpu_ray *rays, int n, float *t,
                                 uint32_t *id, int32_t *hit, cudaStream_t s,
                                 unsigned int *counter = nullptr, unsigned long long *stats = nullptr);

// kd_gpu.cu: the KD tree of KDTree::build on the device, from the build
// vertices and types; node ids breadth-first (scratch kept between builds)
struct KdTree;
struct KdScratch;
KdScratch *kd_scratch_create();
void kd_scratch_destroy(KdScratch *w);
cudaError_t kd_build_gpu(const float *verts, const uint8_t *type, uint32_t n, KdTree &kd, KdScratch &w,
                         cudaStream_t s);

// host helpers shared by the single-scene API and the batch (api.cpp)
int record_error(int code, const std::string &msg);
void make_lights(const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt,
                 std::vector<LightRec> &lights);

}  // namespace ptgpu
