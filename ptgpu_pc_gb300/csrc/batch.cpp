// batch.cpp -- the batched renderer's C ABI (include/ptgpu.h, ptgpu_batch_*).
//
// A batch concatenates its scenes' shapes into one set of device arrays.  The
// build runs each LBVH kernel once over all of them (launch_lbvh_build_seg:
// per-scene centroid bounds and keys, one radix sort whose last pass regroups
// the shapes by scene, per-scene emission tiles); the optional treelet rounds
// then run per scene.  The traversal arrays of all scenes share one node,
// primitive and shape-id space, so a lane of the render kernel only needs its
// scene's record (camera, size, passes, lights, root) next to the shared
// arrays.  Pixels are handed out scene by scene in the order of decreasing
// passes, so the longest pixel chains start first.  The render launch (the
// pixel counter's reset and the kernel) is captured once in a CUDA graph and
// replayed per frame; only the scene records change between frames.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "devbuf.h"
#include "host.h"
#include "lbvh.h"

using namespace ptgpu;

namespace {

struct SceneIn {
    std::vector<ptgpu_shape> shapes;
    uint32_t light_cnt = 0;
    ptgpu_camera cam{};
    int32_t w = 0, h = 0, passes = 1, max_depth = PTGPU_MAX_DEPTH;
    std::vector<uint32_t> seeds;
};

int cuda_fail(cudaError_t e, const char *what) {
    const int code = (e == cudaErrorMemoryAllocation) ? PTGPU_E_OOM : PTGPU_E_DEVICE;
    return record_error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define BK(expr)                                                   \
    do {                                                           \
        cudaError_t e_ = (expr);                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);        \
    } while (0)

}  // namespace

struct ptgpu_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 1;
    int rtl = 0;
    std::vector<SceneIn> scenes;
    // layout of the last build
    std::vector<int32_t> seg_off, tile_off, bb_off;
    std::vector<int64_t> pix_off;       // per scene id
    std::vector<int32_t> order;         // hand-out position -> scene id
    std::vector<BatchScene> recs;       // hand-out order
    std::vector<int64_t> pix_start;     // hand-out offsets
    std::vector<int32_t> current;       // samples accumulated per scene id
    int64_t n_total = 0, px_total = 0;
    double samples = 0.0;
    bool built = false;
    int tree_depth = 0;
    // launch settings
    int block = 128, refill = 0, stack = 64;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float build_ms = 0.f, render_ms = 0.f;
    // device arrays
    DevBuf d_shapes, d_verts, d_type, d_aabbs, d_lb, d_prims0, d_mats, d_lights;
    DevBuf d_btn, d_btl, d_keys, d_keys_alt, d_keys_tmp, d_vals_alt, d_vals_tmp, d_sorted;
    DevBuf d_status, d_state, d_block_bounds, d_arrivals, d_tcount, d_tcost;
    DevBuf d_seg_off, d_tile_off, d_bb_off, d_seg_state, d_depth;
    DevBuf d_nodes, d_prims, d_prim_id, d_recs, d_pix_start;
    DevBuf d_colors, d_pixels, d_seeds, d_seeds0, d_pixctr, d_err;

    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
};

namespace {

RenderArgs render_args(ptgpu_batch *b) {
    RenderArgs a;
    std::memset(&a, 0, sizeof(a));
    a.tv.nodes = b->d_nodes.as<float4>();
    a.tv.nodes4 = nullptr;
    a.tv.prims = b->d_prims.as<float4>();
    a.tv.prim_id = b->d_prim_id.as<int32_t>();
    a.tv.accel = PTGPU_ACCEL_BVH;
    a.tv.error_flags = b->d_err.as<int32_t>();
    a.mats = b->d_mats.as<Material>();
    a.prims0 = b->d_prims0.as<float4>();
    a.lights = b->d_lights.as<LightRec>();
    a.rtl = b->rtl;
    a.colors = b->d_colors.as<ptgpu_vec>();
    a.pixels = b->d_pixels.as<uint32_t>();
    a.seeds = b->d_seeds.as<uint32_t>();
    a.pixel_counter = b->d_pixctr.as<unsigned int>();
    a.refill = b->refill;
    a.scenes = b->d_recs.as<BatchScene>();
    a.pix_start = b->d_pix_start.as<int64_t>();
    a.n_scenes = (int32_t)b->recs.size();
    return a;
}

// scene records with the current start samples (and `passes` if > 0)
cudaError_t upload_recs(ptgpu_batch *b, int passes_override) {
    for (size_t k = 0; k < b->recs.size(); ++k) {
        const int id = b->order[k];
        b->recs[k].start_sample = b->current[id];
        b->recs[k].passes = passes_override > 0 ? passes_override : b->scenes[id].passes;
    }
    return cudaMemcpyAsync(b->d_recs.p, b->recs.data(), b->recs.size() * sizeof(BatchScene),
                           cudaMemcpyHostToDevice, b->stream);
}

int check_render_errors(ptgpu_batch *b) {
    int32_t err = 0;
    BK(cudaMemcpyAsync(&err, b->d_err.p, sizeof(err), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    if (err & 1) return record_error(PTGPU_E_RANGE, "traversal stack overflow");
    return PTGPU_OK;
}

}  // namespace

extern "C" {

int ptgpu_batch_create(int32_t device, uint32_t flags, ptgpu_batch **out) {
    if (!out) return record_error(PTGPU_E_INVAL, "null output");
    *out = nullptr;
    ptgpu_batch *b = new ptgpu_batch();
    b->device = device;
    b->rtl = (flags & PTGPU_FLAG_ARGS_RTL) ? 1 : 0;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = b->d_pixctr.ensure(16);
    if (e == cudaSuccess) e = b->d_err.ensure(16);
    if (e == cudaSuccess) e = b->d_depth.ensure(16);
    if (e != cudaSuccess) {
        const int st = cuda_fail(e, "batch set-up");
        ptgpu_batch_destroy(b);
        return st;
    }
    *out = b;
    return PTGPU_OK;
}

int ptgpu_batch_destroy(ptgpu_batch *b) {
    if (!b) return PTGPU_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    b->drop_graph();
    DevBuf *bufs[] = {&b->d_shapes, &b->d_verts, &b->d_type, &b->d_aabbs, &b->d_lb, &b->d_prims0, &b->d_mats,
                      &b->d_lights, &b->d_btn, &b->d_btl, &b->d_keys, &b->d_keys_alt, &b->d_keys_tmp,
                      &b->d_vals_alt, &b->d_vals_tmp, &b->d_sorted, &b->d_status, &b->d_state,
                      &b->d_block_bounds, &b->d_arrivals, &b->d_tcount, &b->d_tcost, &b->d_seg_off,
                      &b->d_tile_off, &b->d_bb_off, &b->d_seg_state, &b->d_depth, &b->d_nodes,
                      &b->d_prims, &b->d_prim_id, &b->d_recs, &b->d_pix_start, &b->d_colors,
                      &b->d_pixels, &b->d_seeds, &b->d_seeds0, &b->d_pixctr, &b->d_err};
    for (DevBuf *d : bufs) d->release();
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return PTGPU_OK;
}

static int ptgpu_batch_add_body(ptgpu_batch *b, const ptgpu_scene *sc, int32_t *scene_id) {
    if (!b || !sc || !sc->shapes || !sc->seeds) return record_error(PTGPU_E_INVAL, "null argument");
    if ((int)b->scenes.size() >= kMaxSegments)
        return record_error(PTGPU_E_RANGE, "a batch holds at most 256 scenes");
    if (sc->n < 2) return record_error(PTGPU_E_INVAL, "a batched scene needs at least 2 shapes");
    if (sc->width <= 0 || sc->height <= 0 || (int64_t)sc->width * sc->height > (1ll << 30))
        return record_error(PTGPU_E_INVAL, "bad image size");
    if (sc->passes <= 0) return record_error(PTGPU_E_INVAL, "passes must be positive");
    if (sc->max_depth < 0 || sc->max_depth > 1024) return record_error(PTGPU_E_INVAL, "bad max_depth");
    for (uint32_t i = 0; i < sc->n; ++i)
        if (sc->shapes[i].type != PTGPU_SPHERE && sc->shapes[i].type != PTGPU_TRIANGLE)
            return record_error(PTGPU_E_INVAL, "shape " + std::to_string(i) + " has an unknown type");
    SceneIn in;
    in.shapes.assign(sc->shapes, sc->shapes + sc->n);
    in.light_cnt = sc->light_cnt;
    in.cam = sc->camera;
    in.cam.width = (float)sc->width;
    in.cam.height = (float)sc->height;
    update_camera(&in.cam);
    in.w = sc->width;
    in.h = sc->height;
    in.passes = sc->passes;
    in.max_depth = sc->max_depth ? sc->max_depth : PTGPU_MAX_DEPTH;
    in.seeds.assign(sc->seeds, sc->seeds + 2 * (size_t)sc->width * sc->height);
    b->scenes.push_back(std::move(in));
    b->built = false;
    if (scene_id) *scene_id = (int32_t)b->scenes.size() - 1;
    return PTGPU_OK;
}

static int ptgpu_batch_build_body(ptgpu_batch *b, uint32_t flags) {
    if (!b) return record_error(PTGPU_E_INVAL, "null batch");
    if (b->scenes.empty()) return record_error(PTGPU_E_STATE, "no scenes added");
    if (flags & PTGPU_FLAG_MORTON_DELTA) return record_error(PTGPU_E_INVAL, "build flag not supported");
    cudaSetDevice(b->device);
    b->drop_graph();
    b->built = false;
    const int S = (int)b->scenes.size();
    // layout: shapes, tiles, per-level blocks, pixels (all in scene id order)
    b->seg_off.assign(S + 1, 0);
    b->tile_off.assign(S + 1, 0);
    b->bb_off.assign(S + 1, 0);
    b->pix_off.assign(S, 0);
    int64_t n = 0, px = 0, bb = 0;
    int tiles = 0;
    size_t max_n = 0;
    for (int s = 0; s < S; ++s) {
        const SceneIn &in = b->scenes[s];
        b->seg_off[s] = (int32_t)n;
        b->tile_off[s] = tiles;
        b->bb_off[s] = (int32_t)bb;
        b->pix_off[s] = px;
        n += in.shapes.size();
        tiles += emission_tiles((int)in.shapes.size());
        bb += (int64_t)seg_block_bound_count((int)in.shapes.size());
        px += (int64_t)in.w * in.h;
        max_n = std::max(max_n, in.shapes.size());
        if (n >= (1ll << 30)) return record_error(PTGPU_E_RANGE, "more than 2^30 shapes in a batch");
    }
    b->seg_off[S] = (int32_t)n;
    b->tile_off[S] = tiles;
    b->bb_off[S] = (int32_t)bb;
    b->n_total = n;
    b->px_total = px;
    // lights, in scene order
    std::vector<LightRec> lights, sl;
    std::vector<int32_t> light_first(S), light_n(S);
    for (int s = 0; s < S; ++s) {
        const SceneIn &in = b->scenes[s];
        make_lights(in.shapes.data(), (uint32_t)in.shapes.size(), in.light_cnt, sl);
        light_first[s] = (int32_t)lights.size();
        light_n[s] = (int32_t)sl.size();
        lights.insert(lights.end(), sl.begin(), sl.end());
    }
    // device arrays
    const size_t N = (size_t)n;
    BK(b->d_shapes.ensure(N * sizeof(ptgpu_shape)));
    BK(b->d_verts.ensure(N * 9 * sizeof(float)));
    BK(b->d_type.ensure(N));
    BK(b->d_aabbs.ensure(N * 2 * sizeof(float4)));
    BK(b->d_lb.ensure(N * 2 * sizeof(float4)));
    BK(b->d_prims0.ensure(N * 3 * sizeof(float4)));
    BK(b->d_mats.ensure(N * sizeof(Material)));
    BK(b->d_lights.ensure(std::max<size_t>(1, lights.size()) * sizeof(LightRec)));
    BK(b->d_btn.ensure((N - S) * sizeof(ptgpu_bvh_node)));
    BK(b->d_btl.ensure(N * sizeof(ptgpu_bvh_node)));
    BK(b->d_keys.ensure(N * 4));
    BK(b->d_keys_alt.ensure(N * 4));
    BK(b->d_keys_tmp.ensure(N * 4));
    BK(b->d_vals_alt.ensure(N * 4));
    BK(b->d_vals_tmp.ensure(N * 4));
    BK(b->d_sorted.ensure(N * 4));
    BK(b->d_status.ensure(sort_status_words((int)n) * 4));
    BK(b->d_state.ensure(sizeof(BuildState)));
    BK(b->d_block_bounds.ensure((size_t)bb * 6 * sizeof(float)));
    BK(b->d_arrivals.ensure((size_t)bb * sizeof(uint32_t)));
    BK(b->d_seg_off.ensure((S + 1) * sizeof(int32_t)));
    BK(b->d_tile_off.ensure((S + 1) * sizeof(int32_t)));
    BK(b->d_bb_off.ensure((S + 1) * sizeof(int32_t)));
    BK(b->d_seg_state.ensure(S * sizeof(SegState)));
    BK(b->d_nodes.ensure((N - S) * 4 * sizeof(float4)));
    BK(b->d_prims.ensure(N * 3 * sizeof(float4)));
    BK(b->d_prim_id.ensure(N * sizeof(int32_t)));
    BK(b->d_recs.ensure(S * sizeof(BatchScene)));
    BK(b->d_pix_start.ensure((S + 1) * sizeof(int64_t)));
    BK(b->d_colors.ensure((size_t)px * sizeof(ptgpu_vec)));
    BK(b->d_pixels.ensure((size_t)px * sizeof(uint32_t)));
    BK(b->d_seeds.ensure((size_t)px * 2 * sizeof(uint32_t)));
    BK(b->d_seeds0.ensure((size_t)px * 2 * sizeof(uint32_t)));
    // uploads
    for (int s = 0; s < S; ++s) {
        const SceneIn &in = b->scenes[s];
        BK(cudaMemcpyAsync(b->d_shapes.as<ptgpu_shape>() + b->seg_off[s], in.shapes.data(),
                           in.shapes.size() * sizeof(ptgpu_shape), cudaMemcpyHostToDevice, b->stream));
        BK(cudaMemcpyAsync(b->d_seeds.as<uint32_t>() + 2 * b->pix_off[s], in.seeds.data(),
                           in.seeds.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, b->stream));
    }
    BK(cudaMemcpyAsync(b->d_seeds0.p, b->d_seeds.p, (size_t)px * 2 * sizeof(uint32_t),
                       cudaMemcpyDeviceToDevice, b->stream));
    if (!lights.empty())
        BK(cudaMemcpyAsync(b->d_lights.p, lights.data(), lights.size() * sizeof(LightRec),
                           cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_seg_off.p, b->seg_off.data(), (S + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_tile_off.p, b->tile_off.data(), (S + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_bb_off.p, b->bb_off.data(), (S + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
    BK(launch_unpack_shapes(b->d_shapes.as<ptgpu_shape>(), (int)n, b->d_verts.as<float>(),
                            b->d_type.as<uint8_t>(), b->d_prims0.as<float4>(), b->d_mats.as<Material>(),
                            b->stream));
    // the build: every tree in one pass of the LBVH kernels
    LbvhBuffers lb;
    std::memset(&lb, 0, sizeof(lb));
    lb.wait_limit = kDefaultWaitLimit;
    lb.verts = b->d_verts.as<float>();
    lb.type = b->d_type.as<uint8_t>();
    lb.aabbs = b->d_aabbs.as<float4>();
    lb.leaf_bounds = b->d_lb.as<float4>();
    lb.keys = b->d_keys.as<uint32_t>();
    lb.keys_alt = b->d_keys_alt.as<uint32_t>();
    lb.keys_tmp = b->d_keys_tmp.as<uint32_t>();
    lb.vals_alt = b->d_vals_alt.as<int32_t>();
    lb.vals_tmp = b->d_vals_tmp.as<int32_t>();
    lb.sorted = b->d_sorted.as<int32_t>();
    lb.status = b->d_status.as<uint32_t>();
    lb.state = b->d_state.as<BuildState>();
    lb.block_bounds = b->d_block_bounds.as<float>();
    lb.arrivals = b->d_arrivals.as<uint32_t>();
    lb.btn = b->d_btn.as<ptgpu_bvh_node>();
    lb.btl = b->d_btl.as<ptgpu_bvh_node>();
    SegBuild sb;
    sb.seg_off = b->d_seg_off.as<int32_t>();
    sb.tile_off = b->d_tile_off.as<int32_t>();
    sb.bb_off = b->d_bb_off.as<int32_t>();
    sb.seg_state = b->d_seg_state.as<SegState>();
    sb.n_segs = S;
    sb.n_tiles = tiles;
    sb.n_blocks = bb;
    BK(cudaEventRecord(b->ev0, b->stream));
    BK(launch_lbvh_build_seg(lb, (int)n, sb, b->sm_count, b->stream));
    if (flags & PTGPU_FLAG_TREELET) {
        const int sweeps = ((flags >> 8) & 0xF) ? (int)((flags >> 8) & 0xF) : 1;
        BK(b->d_tcount.ensure((size_t)n * sizeof(int)));
        BK(b->d_tcost.ensure((size_t)n * sizeof(float)));
        // every scene's tree in one launch per round
        BK(launch_treelet_seg(lb.btn, lb.btl, b->d_seg_off.as<int32_t>(), S, (int)n, b->d_tcount.as<int>(),
                              b->d_tcost.as<float>(), sweeps, b->stream));
    }
    BK(cudaEventRecord(b->ev1, b->stream));
    uint32_t err_word = 0;
    BK(cudaMemcpyAsync(&err_word, &lb.state->error, sizeof(err_word), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    cudaEventElapsedTime(&b->build_ms, b->ev0, b->ev1);
    if (err_word) return record_error(PTGPU_E_TIMEOUT, "radix sort look-back wait gave up");
    // traversal arrays in the shared index space
    for (int s = 0; s < S; ++s) {
        const int off = b->seg_off[s], ns = b->seg_off[s + 1] - off, nb = off - s;
        BK(launch_abi_to_trace(lb.btn + nb, lb.btl + off, ns, b->d_prims0.as<float4>() + 3 * (size_t)off,
                               b->d_nodes.as<float4>() + 4 * (size_t)nb,
                               b->d_prims.as<float4>() + 3 * (size_t)off,
                               b->d_prim_id.as<int32_t>() + off, b->stream, nb, off));
    }
    BK(launch_tree_depth(lb.btn, lb.btl, b->d_seg_off.as<int32_t>(), S, (int)n, b->d_depth.as<int>(),
                         b->stream));
    // scene records in hand-out order: most passes first, then most pixels
    b->order.resize(S);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
        const SceneIn &p = b->scenes[x], &q = b->scenes[y];
        if (p.passes != q.passes) return p.passes > q.passes;
        return (int64_t)p.w * p.h > (int64_t)q.w * q.h;
    });
    b->recs.assign(S, BatchScene{});
    b->pix_start.assign(S + 1, 0);
    b->samples = 0.0;
    for (int k = 0; k < S; ++k) {
        const int s = b->order[k];
        const SceneIn &in = b->scenes[s];
        BatchScene &r = b->recs[k];
        std::memset(&r, 0, sizeof(r));
        r.cam = in.cam;
        r.width = in.w;
        r.height = in.h;
        r.passes = in.passes;
        r.max_depth = in.max_depth;
        r.start_sample = 0;
        r.root = b->seg_off[s] - s;
        r.n_shapes = (int32_t)in.shapes.size();
        r.skip = b->seg_off[s + 1] - 1;
        r.shape0 = b->seg_off[s];
        r.light_first = light_first[s];
        r.n_lights = light_n[s];
        r.pix_off = b->pix_off[s];
        b->pix_start[k + 1] = b->pix_start[k] + (int64_t)in.w * in.h;
        b->samples += (double)in.w * in.h * in.passes;
    }
    BK(cudaMemcpyAsync(b->d_recs.p, b->recs.data(), S * sizeof(BatchScene), cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(b->d_pix_start.p, b->pix_start.data(), (S + 1) * sizeof(int64_t),
                       cudaMemcpyHostToDevice, b->stream));
    BK(launch_fill_roots(b->d_recs.as<BatchScene>(), S, lb.btn, b->stream));
    // the records with their root bounds, as later frames upload them
    BK(cudaMemcpyAsync(b->recs.data(), b->d_recs.p, S * sizeof(BatchScene), cudaMemcpyDeviceToHost,
                       b->stream));
    int depth = 0;
    BK(cudaMemcpyAsync(&depth, b->d_depth.p, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaMemsetAsync(b->d_err.p, 0, 16, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    b->tree_depth = depth;
    b->stack = render_stack_for_depth(depth);
    b->current.assign(S, 0);
    b->built = true;
    return PTGPU_OK;
}

static int render_once(ptgpu_batch *b, bool use_graph) {
    RenderArgs a = render_args(b);
    const int grid = render_batch_grid(b->block, b->stack, 0);
    if (grid <= 0) return record_error(PTGPU_E_DEVICE, "no resident CTA for the render kernel");
    if (!use_graph) {
        BK(cudaEventRecord(b->ev0, b->stream));
        BK(launch_render_batch(a, b->block, b->stack, grid, b->stream));
        BK(cudaEventRecord(b->ev1, b->stream));
        return PTGPU_OK;
    }
    if (!b->exec) {
        BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = launch_render_batch(a, b->block, b->stack, grid, b->stream);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(e, "render capture"); }
        if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
        b->graph = g;
        BK(cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    BK(cudaEventRecord(b->ev0, b->stream));
    BK(cudaGraphLaunch(b->exec, b->stream));
    BK(cudaEventRecord(b->ev1, b->stream));
    return PTGPU_OK;
}

int ptgpu_batch_render(ptgpu_batch *b) {
    if (!b) return record_error(PTGPU_E_INVAL, "null batch");
    if (!b->built) return record_error(PTGPU_E_STATE, "build the batch first");
    cudaSetDevice(b->device);
    BK(upload_recs(b, 0));
    int st = render_once(b, true);
    if (st) return st;
    BK(cudaStreamSynchronize(b->stream));
    cudaEventElapsedTime(&b->render_ms, b->ev0, b->ev1);
    st = check_render_errors(b);
    if (st) return st;
    for (size_t s = 0; s < b->scenes.size(); ++s) b->current[s] += b->scenes[s].passes;
    return PTGPU_OK;
}

int ptgpu_batch_reset(ptgpu_batch *b) {
    if (!b) return record_error(PTGPU_E_INVAL, "null batch");
    std::fill(b->current.begin(), b->current.end(), 0);
    return PTGPU_OK;
}

int ptgpu_batch_tune(ptgpu_batch *b) {
    if (!b) return record_error(PTGPU_E_INVAL, "null batch");
    if (!b->built) return record_error(PTGPU_E_STATE, "build the batch first");
    cudaSetDevice(b->device);
    // the render kernel is compiled for at most 128 threads per CTA
    static const int kBlocks[] = {64, 96, 128};
    static const int kRefill[] = {16, 20, 24};
    std::fill(b->current.begin(), b->current.end(), 0);
    BK(upload_recs(b, 1));                     // one pass per scene per trial
    float best = 1e30f;
    int best_block = b->block, best_refill = b->refill;
    for (int rep = 0; rep < 2; ++rep) {        // the first round also warms up
        for (int blk : kBlocks) {
            for (int rf : kRefill) {
                b->block = blk;
                b->refill = rf;
                BK(cudaMemcpyAsync(b->d_seeds.p, b->d_seeds0.p, (size_t)b->px_total * 2 * sizeof(uint32_t),
                                   cudaMemcpyDeviceToDevice, b->stream));
                int st = render_once(b, false);
                if (st) return st;
                BK(cudaStreamSynchronize(b->stream));
                float ms = 0.f;
                cudaEventElapsedTime(&ms, b->ev0, b->ev1);
                if (rep == 1 && ms < best) { best = ms; best_block = blk; best_refill = rf; }
            }
        }
    }
    b->block = best_block;
    b->refill = best_refill;
    b->drop_graph();
    BK(cudaMemcpyAsync(b->d_seeds.p, b->d_seeds0.p, (size_t)b->px_total * 2 * sizeof(uint32_t),
                       cudaMemcpyDeviceToDevice, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    return check_render_errors(b);
}

int ptgpu_batch_get_pixels(ptgpu_batch *b, int32_t scene, uint32_t *pixels) {
    if (!b || !pixels) return record_error(PTGPU_E_INVAL, "null argument");
    if (!b->built || scene < 0 || scene >= (int)b->scenes.size())
        return record_error(PTGPU_E_INVAL, "no such scene in the built batch");
    const SceneIn &in = b->scenes[scene];
    BK(cudaMemcpyAsync(pixels, b->d_pixels.as<uint32_t>() + b->pix_off[scene],
                       (size_t)in.w * in.h * sizeof(uint32_t), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    return PTGPU_OK;
}

int ptgpu_batch_get_colors(ptgpu_batch *b, int32_t scene, ptgpu_vec *colors) {
    if (!b || !colors) return record_error(PTGPU_E_INVAL, "null argument");
    if (!b->built || scene < 0 || scene >= (int)b->scenes.size())
        return record_error(PTGPU_E_INVAL, "no such scene in the built batch");
    const SceneIn &in = b->scenes[scene];
    BK(cudaMemcpyAsync(colors, b->d_colors.as<ptgpu_vec>() + b->pix_off[scene],
                       (size_t)in.w * in.h * sizeof(ptgpu_vec), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    return PTGPU_OK;
}

int ptgpu_batch_get_bvh(ptgpu_batch *b, int32_t scene, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl) {
    if (!b || !btn || !btl) return record_error(PTGPU_E_INVAL, "null argument");
    if (!b->built || scene < 0 || scene >= (int)b->scenes.size())
        return record_error(PTGPU_E_INVAL, "no such scene in the built batch");
    const int off = b->seg_off[scene], ns = b->seg_off[scene + 1] - off;
    BK(cudaMemcpyAsync(btn, b->d_btn.as<ptgpu_bvh_node>() + (off - scene),
                       (size_t)(ns - 1) * sizeof(ptgpu_bvh_node), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaMemcpyAsync(btl, b->d_btl.as<ptgpu_bvh_node>() + off, (size_t)ns * sizeof(ptgpu_bvh_node),
                       cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    return PTGPU_OK;
}

int ptgpu_batch_info_get(ptgpu_batch *b, ptgpu_batch_info *info) {
    if (!b || !info) return record_error(PTGPU_E_INVAL, "null argument");
    std::memset(info, 0, sizeof(*info));
    info->build_ms = b->build_ms;
    info->render_ms = b->render_ms;
    info->samples = b->samples;
    info->block = b->block;
    info->refill = b->refill;
    info->stack = b->stack;
    info->tree_depth = b->tree_depth;
    info->shapes = b->n_total;
    return PTGPU_OK;
}

}  // extern "C"

// C entry points: no C++ exception crosses the C ABI
int ptgpu_batch_add(ptgpu_batch *b, const ptgpu_scene *sc, int32_t *scene_id) {
    try {
        return ptgpu_batch_add_body(b, sc, scene_id);
    } catch (const std::bad_alloc &) {
        return record_error(PTGPU_E_OOM, "out of host memory");
    } catch (const std::exception &e) {
        return record_error(PTGPU_E_INVAL, std::string("unexpected error: ") + e.what());
    }
}

int ptgpu_batch_build(ptgpu_batch *b, uint32_t flags) {
    try {
        return ptgpu_batch_build_body(b, flags);
    } catch (const std::bad_alloc &) {
        return record_error(PTGPU_E_OOM, "out of host memory");
    } catch (const std::exception &e) {
        return record_error(PTGPU_E_INVAL, std::string("unexpected error: ") + e.what());
    }
}
