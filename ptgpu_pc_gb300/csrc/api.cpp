// api.cpp -- the C ABI (include/ptgpu.h): context, scene, builds, rendering.
//
// The context replaces the reference's process globals (smallptGPU.cpp:108-
// 119, displayfunc.cpp:85-98): shapes, light count, camera, seeds, the
// accumulation buffer and the acceleration structure all live in one object
// that owns its device memory and stream.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "devbuf.h"
#include "host.h"
#include "ingest.h"
#include "lbvh.h"

using namespace ptgpu;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    int code = (e == cudaErrorMemoryAllocation) ? PTGPU_E_OOM : PTGPU_E_DEVICE;
    return fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(expr)                                                   \
    do {                                                           \
        cudaError_t e_ = (expr);                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);        \
    } while (0)

bool viszero(const ptgpu_vec &v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }

}  // namespace

namespace ptgpu {
// lets entry points outside this file report through ptgpu_last_error()
int record_error(int code, const std::string &msg) { return fail(code, msg); }

// SampleLights' emitters: the first light_cnt shapes with non-zero emission,
// in index order
void make_lights(const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt,
                 std::vector<LightRec> &lights) {
    lights.clear();
    for (uint32_t i = 0; i < n && lights.size() < light_cnt; ++i) {
        const ptgpu_shape &s = shapes[i];
        if (viszero(s.e)) continue;
        LightRec L;
        std::memset(&L, 0, sizeof(L));
        if (s.type == PTGPU_TRIANGLE) {
            const ptgpu_triangle &t = s.g.t;
            int32_t tt = PTGPU_TRIANGLE; float tf; std::memcpy(&tf, &tt, 4);
            L.a = make_float4(t.p1.x, t.p1.y, t.p1.z, tf);
            L.b = make_float4(t.p2.x - t.p1.x, t.p2.y - t.p1.y, t.p2.z - t.p1.z, s.area);
            L.c = make_float4(t.p3.x - t.p1.x, t.p3.y - t.p1.y, t.p3.z - t.p1.z, 0.f);
        } else {
            int32_t tt = PTGPU_SPHERE; float tf; std::memcpy(&tf, &tt, 4);
            L.a = make_float4(s.g.s.p.x, s.g.s.p.y, s.g.s.p.z, tf);
            L.b = make_float4(s.g.s.rad, 0.f, 0.f, s.area);
        }
        L.e = make_float4(s.e.x, s.e.y, s.e.z, 0.f);
        lights.push_back(L);
    }
}
}  // namespace ptgpu

struct ptgpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sm_count = 1;
    int max_depth = PTGPU_MAX_DEPTH;
    int accel_cfg = PTGPU_ACCEL_BVH;
    int block = 128;
    int flags = 0;
    uint32_t wait_limit = kDefaultWaitLimit;   // look-back polls before E_TIMEOUT
    // scene
    // the scene's shape records: d_shapes holds them as set (never modified);
    // the host copy is made from it only when a call needs one
    std::vector<ptgpu_shape> h_shapes;
    bool host_shapes = false;            // h_shapes holds the scene
    DevBuf d_export;                     // the records with a BVH build's index / morton / b
    bool export_ready = false;           // d_export holds them
    bool kd_indexed = false;             // a KD build numbered the host copy's shapes
    IngestScratch ingest;
    uint32_t n = 0, light_cnt = 0;
    int n_lights = 0;
    bool all_tri = true;
    DevBuf d_shapes, d_verts, d_type, d_prims0, d_mats, d_lights;
    bool shapes_exported = false;
    // acceleration structure
    int accel_built = -1;
    bool bvh_valid = false;
    DevBuf d_btn, d_btl, d_keys, d_keys_alt, d_keys_tmp, d_vals_alt, d_vals_tmp, d_sorted;
    DevBuf d_status, d_state, d_block_bounds, d_arrivals, d_tcount, d_tcost, d_aabbs;
    DevBuf d_nodes, d_nodes4, d_prims, d_prim_id, d_root_box, d_identity;
    int n_internal = 0;
    bool wide = false;
    int32_t root_first = 0, root_count = 0;
    KdTree kd;
    KdScratch *kd_scratch = nullptr;
    bool kd_valid = false;
    // rendering
    int w = 0, h = 0;
    DevBuf d_colors, d_pixels, d_seeds, d_err, d_pixctr, d_wf;
    DevBuf d_cost, d_order, d_order_scr;   // per-pixel work, next hand-out order
    DevBuf d_img, d_rowoff;                 // an encoded image, its PPM row offsets
    bool order_valid = false;
    uint32_t *h_pixels = nullptr;
    int current_sample = 0;
    ptgpu_camera cam{};
    bool cam_set = false;
    // queries
    DevBuf d_rays, d_t, d_id, d_hit;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_build_ms = 0.f;
    int rtl = 0;
    int rr_depth = 0;     // ptgpu_config.rr_depth
};

static TraceView make_view(ptgpu_ctx *c) {
    TraceView tv;
    std::memset(&tv, 0, sizeof(tv));
    tv.n_shapes = (int32_t)c->n;
    tv.error_flags = c->d_err.as<int32_t>();
    if (c->accel_built == PTGPU_ACCEL_NONE || (c->accel_built == PTGPU_ACCEL_BVH && c->n == 1)) {
        tv.accel = PTGPU_ACCEL_NONE;
        tv.prims = c->d_prims0.as<float4>();
        tv.prim_id = c->d_identity.as<int32_t>();
        return tv;
    }
    tv.accel = c->accel_built;
    tv.nodes = c->d_nodes.as<float4>();
    tv.nodes4 = (c->wide && c->root_count == 0 && c->n_internal > 0) ? c->d_nodes4.as<float4>() : nullptr;
    tv.prims = c->d_prims.as<float4>();
    tv.prim_id = c->d_prim_id.as<int32_t>();
    tv.root_first = c->root_first;
    tv.root_count = c->root_count;
    tv.root_box = c->d_root_box.as<float>();
    return tv;
}

extern "C" {

int ptgpu_abi_version(void) { return PTGPU_ABI_VERSION; }

const char *ptgpu_last_error(void) { return g_last_error.c_str(); }

const char *ptgpu_status_string(int s) {
    switch (s) {
    case PTGPU_OK: return "ok";
    case PTGPU_E_INVAL: return "invalid argument";
    case PTGPU_E_OOM: return "out of memory";
    case PTGPU_E_DEVICE: return "device error";
    case PTGPU_E_TIMEOUT: return "device wait timed out";
    case PTGPU_E_IO: return "scene i/o error";
    case PTGPU_E_RANGE: return "result does not fit the reference layout";
    case PTGPU_E_STATE: return "call out of order";
    case PTGPU_E_CANCELED: return "request cancelled";
    default: return "unknown status";
    }
}

int ptgpu_make_seeds(uint64_t master, uint32_t *seeds, uint32_t count) {
    if (!seeds && count) return fail(PTGPU_E_INVAL, "null seed buffer");
    make_seeds(master, seeds, count);
    return PTGPU_OK;
}

int ptgpu_update_camera(ptgpu_camera *cam) {
    if (!cam) return fail(PTGPU_E_INVAL, "null camera");
    update_camera(cam);
    return PTGPU_OK;
}

int ptgpu_create(const ptgpu_config *cfg, ptgpu_ctx **out) {
    if (!cfg || !out) return fail(PTGPU_E_INVAL, "null config or output");
    if (cfg->width <= 0 || cfg->height <= 0 || (int64_t)cfg->width * cfg->height > (1ll << 30))
        return fail(PTGPU_E_INVAL, "width and height must be positive");
    if (cfg->accel < 0 || cfg->accel > 2) return fail(PTGPU_E_INVAL, "accel must be 0, 1 or 2");
    if (cfg->max_depth < 0 || cfg->max_depth > 1024) return fail(PTGPU_E_INVAL, "bad max_depth");
    if (cfg->rr_depth < 0) return fail(PTGPU_E_INVAL, "rr_depth must be >= 0");
    if (cfg->rr_depth > 0 && (cfg->flags & PTGPU_FLAG_WAVEFRONT))
        return fail(PTGPU_E_INVAL, "rr_depth applies to the lane tracer, not PTGPU_FLAG_WAVEFRONT");
    *out = nullptr;
    ptgpu_ctx *c = new ptgpu_ctx();
    c->device = cfg->device;
    c->accel_cfg = cfg->accel;
    c->max_depth = cfg->max_depth ? cfg->max_depth : PTGPU_MAX_DEPTH;
    c->block = cfg->block_size > 0 ? cfg->block_size : 128;
    c->flags = cfg->flags;
    c->rtl = (cfg->flags & PTGPU_FLAG_ARGS_RTL) ? 1 : 0;
    c->rr_depth = cfg->rr_depth;
    c->wide = (cfg->flags & PTGPU_FLAG_WIDE_TRAVERSAL) ? true : false;
    c->w = cfg->width;
    c->h = cfg->height;
    auto bail = [&](int code) { ptgpu_destroy(c); return code; };
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaSetDevice"));
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
    if (cfg->stream) {
        c->stream = (cudaStream_t)cfg->stream;
    } else {
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
        c->own_stream = true;
    }
    if ((e = cudaEventCreate(&c->ev0)) != cudaSuccess) return bail(cuda_fail(e, "cudaEventCreate"));
    if ((e = cudaEventCreate(&c->ev1)) != cudaSuccess) return bail(cuda_fail(e, "cudaEventCreate"));
    const size_t npx = (size_t)c->w * c->h;
    if ((e = c->d_colors.ensure(npx * sizeof(ptgpu_vec))) != cudaSuccess) return bail(cuda_fail(e, "alloc colors"));
    if ((e = c->d_pixels.ensure(npx * sizeof(uint32_t))) != cudaSuccess) return bail(cuda_fail(e, "alloc pixels"));
    if ((e = c->d_seeds.ensure(npx * 2 * sizeof(uint32_t))) != cudaSuccess) return bail(cuda_fail(e, "alloc seeds"));
    if ((e = c->d_err.ensure(16)) != cudaSuccess) return bail(cuda_fail(e, "alloc error word"));
    if ((e = c->d_pixctr.ensure(16)) != cudaSuccess) return bail(cuda_fail(e, "alloc pixel counter"));
    if ((e = cudaMallocHost(&c->h_pixels, npx * sizeof(uint32_t))) != cudaSuccess)
        return bail(cuda_fail(e, "alloc pinned pixels"));
    cudaMemsetAsync(c->d_err.p, 0, 16, c->stream);
    cudaMemsetAsync(c->d_colors.p, 0, npx * sizeof(ptgpu_vec), c->stream);
    std::vector<uint32_t> seeds(npx * 2);
    make_seeds(1, seeds.data(), (uint32_t)seeds.size());
    e = cudaMemcpyAsync(c->d_seeds.p, seeds.data(), seeds.size() * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "upload seeds"));
    *out = c;
    return PTGPU_OK;
}

int ptgpu_destroy(ptgpu_ctx *c) {
    if (!c) return PTGPU_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    DevBuf *bufs[] = {&c->d_shapes, &c->d_verts, &c->d_type, &c->d_prims0, &c->d_mats, &c->d_lights,
                      &c->d_btn, &c->d_btl, &c->d_keys, &c->d_keys_alt, &c->d_keys_tmp, &c->d_vals_alt,
                      &c->d_vals_tmp, &c->d_sorted, &c->d_status, &c->d_state, &c->d_block_bounds, &c->d_arrivals,
                      &c->d_tcount, &c->d_tcost, &c->d_aabbs,
                      &c->d_nodes, &c->d_nodes4, &c->d_prims, &c->d_prim_id, &c->d_root_box, &c->d_identity,
                      &c->d_colors, &c->d_pixels, &c->d_seeds, &c->d_err, &c->d_pixctr, &c->d_wf, &c->d_rays, &c->d_t,
                      &c->d_cost, &c->d_order, &c->d_order_scr, &c->d_export,
                      &c->d_id, &c->d_hit};
    for (DevBuf *b : bufs) b->release();
    c->ingest.release();
    kd_scratch_destroy(c->kd_scratch);
    if (c->h_pixels) cudaFreeHost(c->h_pixels);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return PTGPU_OK;
}

int ptgpu_get_stream(ptgpu_ctx *c, void **stream) {
    if (!c || !stream) return fail(PTGPU_E_INVAL, "null argument");
    *stream = (void *)c->stream;
    return PTGPU_OK;
}

// Device arrays of a scene of n shapes with n_lights light records.
static int alloc_scene(ptgpu_ctx *c, uint32_t n, int n_lights) {
    CK(c->d_shapes.ensure((size_t)n * sizeof(ptgpu_shape)));
    CK(c->d_verts.ensure((size_t)n * 9 * sizeof(float)));
    CK(c->d_type.ensure((size_t)n));
    CK(c->d_prims0.ensure((size_t)n * 3 * sizeof(float4)));
    CK(c->d_mats.ensure((size_t)n * sizeof(Material)));
    CK(c->d_lights.ensure((size_t)n_lights * sizeof(LightRec)));
    CK(c->d_identity.ensure((size_t)n * sizeof(int32_t)));
    return PTGPU_OK;
}

// The rest of a scene upload once d_shapes and d_lights hold it: the build
// and traversal arrays derived from the shapes, and a fresh accumulation.
static int finish_scene(ptgpu_ctx *c, uint32_t n, uint32_t light_cnt, int n_lights, bool all_tri) {
    c->n = n;
    c->light_cnt = light_cnt;
    c->n_lights = n_lights;
    c->all_tri = all_tri;
    std::vector<int32_t> ident(n);
    for (uint32_t i = 0; i < n; ++i) ident[i] = (int32_t)i;
    CK(cudaMemcpyAsync(c->d_identity.p, ident.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
    CK(launch_unpack_shapes(c->d_shapes.as<ptgpu_shape>(), (int)n, c->d_verts.as<float>(),
                            c->d_type.as<uint8_t>(), c->d_prims0.as<float4>(), c->d_mats.as<Material>(),
                            c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->accel_built = -1;
    c->bvh_valid = false;
    c->kd_valid = false;
    c->shapes_exported = false;
    c->export_ready = false;
    c->kd_indexed = false;
    c->current_sample = 0;
    return PTGPU_OK;
}

static int ptgpu_set_shapes_body(ptgpu_ctx *c, const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt) {
    if (!c || (!shapes && n)) return fail(PTGPU_E_INVAL, "null argument");
    if (n == 0) return fail(PTGPU_E_INVAL, "a scene needs at least one shape");
    if (n >= (1u << 30)) return fail(PTGPU_E_INVAL, "too many shapes (limit 2^30-1)");
    for (uint32_t i = 0; i < n; ++i)
        if (shapes[i].type != PTGPU_SPHERE && shapes[i].type != PTGPU_TRIANGLE)
            return fail(PTGPU_E_INVAL, "shape " + std::to_string(i) + " has an unknown type");
    cudaSetDevice(c->device);
    c->h_shapes.clear();
    c->h_shapes.shrink_to_fit();
    c->host_shapes = false;
    bool all_tri = true;
    for (uint32_t i = 0; i < n; ++i) if (shapes[i].type != PTGPU_TRIANGLE) { all_tri = false; break; }
    // emitters visited by SampleLights: the first light_cnt in index order
    std::vector<LightRec> lights;
    make_lights(shapes, n, light_cnt, lights);
    int st = alloc_scene(c, n, (int)lights.size());
    if (st) return st;
    CK(cudaMemcpyAsync(c->d_shapes.p, shapes, (size_t)n * sizeof(ptgpu_shape), cudaMemcpyHostToDevice, c->stream));
    if (!lights.empty())
        CK(cudaMemcpyAsync(c->d_lights.p, lights.data(), lights.size() * sizeof(LightRec), cudaMemcpyHostToDevice, c->stream));
    return finish_scene(c, n, light_cnt, (int)lights.size(), all_tri);
}

// The host copy of the scene, for the calls that need one (ptgpu_get_shapes
// without a BVH, the host KD build): the records as set, copied from the
// device once, with the numbering a KD build gives them.
static int ensure_host_shapes(ptgpu_ctx *c) {
    if (c->host_shapes) return PTGPU_OK;
    c->h_shapes.resize(c->n);
    CK(cudaMemcpyAsync(c->h_shapes.data(), c->d_shapes.p, (size_t)c->n * sizeof(ptgpu_shape),
                       cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (c->kd_indexed)
        for (uint32_t i = 0; i < c->n; ++i) { c->h_shapes[i].index = (int32_t)i; c->h_shapes[i].morton_code = 0; }
    c->host_shapes = true;
    return PTGPU_OK;
}

int ptgpu_get_shape_count(ptgpu_ctx *c, uint32_t *n, uint32_t *light_cnt) {
    if (!c) return fail(PTGPU_E_INVAL, "null context");
    if (n) *n = c->n;
    if (light_cnt) *light_cnt = c->light_cnt;
    return PTGPU_OK;
}

static int ptgpu_get_shapes_body(ptgpu_ctx *c, ptgpu_shape *out, uint32_t n) {
    if (!c || !out) return fail(PTGPU_E_INVAL, "null argument");
    if (n != c->n) return fail(PTGPU_E_INVAL, "shape count mismatch");
    if (c->accel_built == PTGPU_ACCEL_BVH && c->bvh_valid && c->d_keys.p) {
        cudaSetDevice(c->device);
        if (!c->shapes_exported) {
            CK(c->d_export.ensure((size_t)n * sizeof(ptgpu_shape)));
            CK(launch_export_shapes(c->d_shapes.as<ptgpu_shape>(), c->d_export.as<ptgpu_shape>(),
                                    c->d_verts.as<float>(), c->d_type.as<uint8_t>(), c->d_keys.as<uint32_t>(),
                                    (int)n, c->stream));
            c->shapes_exported = true;
            c->export_ready = true;
        }
        const void *src = c->export_ready ? c->d_export.p : c->d_shapes.p;
        CK(cudaMemcpyAsync(out, src, (size_t)n * sizeof(ptgpu_shape), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        return PTGPU_OK;
    }
    int st = ensure_host_shapes(c);
    if (st) return st;
    std::memcpy(out, c->h_shapes.data(), (size_t)n * sizeof(ptgpu_shape));
    return PTGPU_OK;
}

static int ptgpu_read_scene_body(ptgpu_ctx *c, const char *path, int32_t *walllight) {
    if (!c || !path) return fail(PTGPU_E_INVAL, "null argument");
    LoadedScene sc;
    std::string err;
    int st = read_scene(path, c->w, c->h, sc, err);
    if (st != PTGPU_OK) return fail(st, err);
    if (sc.walllight) add_wall_light(sc);      // main(): if (walllight) AddWallLight()
    if (walllight) *walllight = sc.walllight ? 1 : 0;
    st = ptgpu_set_shapes(c, sc.shapes.data(), (uint32_t)sc.shapes.size(), sc.light_cnt);
    if (st != PTGPU_OK) return st;
    return ptgpu_set_camera(c, &sc.camera);
}

static int ptgpu_stream_scene_body(ptgpu_ctx *c, const char *path, int32_t *walllight) {
    if (!c || !path) return fail(PTGPU_E_INVAL, "null argument");
    CompactScene sc;
    std::string err;
    int st = read_scene_compact(path, c->w, c->h, sc, err);
    if (st != PTGPU_OK) return fail(st, err);
    if (sc.walllight) add_wall_light(sc);      // main(): if (walllight) AddWallLight()
    if (walllight) *walllight = sc.walllight ? 1 : 0;
    const int64_t n = sc.count();
    if (n == 0) return fail(PTGPU_E_INVAL, "a scene needs at least one shape");
    if (n >= (1 << 30)) return fail(PTGPU_E_INVAL, "too many shapes (limit 2^30-1)");
    cudaSetDevice(c->device);
    const uint32_t n_lights = compact_light_count(sc);
    st = alloc_scene(c, (uint32_t)n, (int)n_lights);
    if (st) return st;
    c->h_shapes.clear();
    c->h_shapes.shrink_to_fit();
    c->host_shapes = false;
    CK(ingest_compact(sc, c->d_shapes.as<ptgpu_shape>(), c->d_lights.as<LightRec>(), c->ingest, c->stream));
    st = finish_scene(c, (uint32_t)n, sc.light_cnt, (int)n_lights, compact_all_triangles(sc));
    if (st != PTGPU_OK) return st;
    return ptgpu_set_camera(c, &sc.camera);
}

int ptgpu_set_camera(ptgpu_ctx *c, const ptgpu_camera *cam) {
    if (!c || !cam) return fail(PTGPU_E_INVAL, "null argument");
    c->cam = *cam;
    c->cam.width = (float)c->w;
    c->cam.height = (float)c->h;
    update_camera(&c->cam);
    c->cam_set = true;
    c->current_sample = 0;
    return PTGPU_OK;
}

int ptgpu_get_camera(ptgpu_ctx *c, ptgpu_camera *cam) {
    if (!c || !cam) return fail(PTGPU_E_INVAL, "null argument");
    *cam = c->cam;
    return PTGPU_OK;
}

static int ensure_bvh_buffers(ptgpu_ctx *c) {
    const size_t n = c->n;
    CK(c->d_btn.ensure((n > 1 ? n - 1 : 1) * sizeof(ptgpu_bvh_node)));
    CK(c->d_btl.ensure(n * sizeof(ptgpu_bvh_node)));
    CK(c->d_aabbs.ensure(n * 2 * sizeof(float4)));
    CK(c->d_keys.ensure(n * 4));
    CK(c->d_keys_alt.ensure(n * 4));
    CK(c->d_keys_tmp.ensure(n * 4));
    CK(c->d_vals_alt.ensure(n * 4));
    CK(c->d_vals_tmp.ensure(n * 4));
    CK(c->d_sorted.ensure(n * 4));
    CK(c->d_status.ensure(sort_status_words((int)n) * 4));
    CK(c->d_state.ensure(sizeof(BuildState)));
    CK(c->d_block_bounds.ensure(block_bound_count((int)n) * 6 * sizeof(float)));
    CK(c->d_arrivals.ensure(block_bound_count((int)n) * sizeof(uint32_t)));
    return PTGPU_OK;
}

static int prepare_wide(ptgpu_ctx *c) {
    if (!c->wide || c->n_internal <= 0) return PTGPU_OK;   // 4-wide nodes only when traversed
    CK(c->d_nodes4.ensure((size_t)c->n_internal * 8 * sizeof(float4)));
    CK(launch_collapse4(c->d_nodes.as<float4>(), c->n_internal, c->d_nodes4.as<float4>(), c->stream));
    return PTGPU_OK;
}

static int prepare_bvh_trace(ptgpu_ctx *c) {
    const size_t n = c->n;
    CK(c->d_nodes.ensure((n > 1 ? n - 1 : 1) * 4 * sizeof(float4)));
    CK(c->d_prims.ensure(n * 3 * sizeof(float4)));
    CK(c->d_prim_id.ensure(n * 4));
    CK(c->d_root_box.ensure(6 * sizeof(float)));
    CK(launch_abi_to_trace(c->d_btn.as<ptgpu_bvh_node>(), c->d_btl.as<ptgpu_bvh_node>(), (int)n,
                           c->d_prims0.as<float4>(), c->d_nodes.as<float4>(), c->d_prims.as<float4>(),
                           c->d_prim_id.as<int32_t>(), c->stream));
    const ptgpu_bvh_node *root = n > 1 ? c->d_btn.as<ptgpu_bvh_node>() : c->d_btl.as<ptgpu_bvh_node>();
    CK(cudaMemcpyAsync(c->d_root_box.p, &root->bound, 6 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    c->root_first = 0;
    c->root_count = n > 1 ? 0 : 1;
    c->n_internal = n > 1 ? (int)(n - 1) : 0;
    return prepare_wide(c);
}

static int ptgpu_build_body(ptgpu_ctx *c, int32_t accel, uint32_t flags) {
    if (!c) return fail(PTGPU_E_INVAL, "null context");
    if (c->n == 0) return fail(PTGPU_E_STATE, "no shapes set");
    if (accel < 0 || accel > 2) return fail(PTGPU_E_INVAL, "accel must be 0, 1 or 2");
    if (flags & PTGPU_FLAG_MORTON_DELTA)
        return fail(PTGPU_E_INVAL, "PTGPU_FLAG_MORTON_DELTA is reserved: the build keeps the index-prefix topology");
    if ((flags & PTGPU_FLAG_TREELET) && accel != PTGPU_ACCEL_BVH)
        return fail(PTGPU_E_INVAL, "treelet restructuring applies to the BVH only");
    cudaSetDevice(c->device);
    c->accel_built = -1;
    c->current_sample = 0;
    if (accel == PTGPU_ACCEL_NONE) {
        c->accel_built = PTGPU_ACCEL_NONE;
        c->last_build_ms = 0.f;
        return PTGPU_OK;
    }
    if (accel == PTGPU_ACCEL_BVH) {
        int st = ensure_bvh_buffers(c);
        if (st) return st;
        LbvhBuffers b;
        b.verts = c->d_verts.as<float>();
        b.type = c->d_type.as<uint8_t>();
        b.aabbs = c->d_aabbs.as<float4>();
        b.leaf_bounds = nullptr;                 // batched builds only
        b.keys = c->d_keys.as<uint32_t>();
        b.keys_alt = c->d_keys_alt.as<uint32_t>();
        b.keys_tmp = c->d_keys_tmp.as<uint32_t>();
        b.vals_alt = c->d_vals_alt.as<int32_t>();
        b.vals_tmp = c->d_vals_tmp.as<int32_t>();
        b.sorted = c->d_sorted.as<int32_t>();
        b.status = c->d_status.as<uint32_t>();
        b.state = c->d_state.as<BuildState>();
        b.block_bounds = c->d_block_bounds.as<float>();
        b.arrivals = c->d_arrivals.as<uint32_t>();
        b.btn = c->d_btn.as<ptgpu_bvh_node>();
        b.btl = c->d_btl.as<ptgpu_bvh_node>();
        b.wait_limit = c->wait_limit;
        CK(cudaEventRecord(c->ev0, c->stream));
        CK(launch_lbvh_build(b, (int)c->n, c->all_tri ? 1 : 0, c->sm_count, c->stream));
        if (flags & PTGPU_FLAG_TREELET) {
            CK(c->d_tcount.ensure((c->n > 1 ? c->n - 1 : 1) * sizeof(int)));
            CK(c->d_tcost.ensure((c->n > 1 ? c->n - 1 : 1) * sizeof(float)));
            const int sweeps = (flags >> 8) & 0xF;
            CK(launch_treelet(b.btn, b.btl, (int)c->n, c->d_tcount.as<int>(), c->d_tcost.as<float>(),
                              sweeps > 0 ? sweeps : 1, c->stream));
        }
        CK(cudaEventRecord(c->ev1, c->stream));
        BuildState hs;
        CK(cudaMemcpyAsync(&hs, c->d_state.p, sizeof(hs), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        cudaEventElapsedTime(&c->last_build_ms, c->ev0, c->ev1);
        if (hs.error) return fail(PTGPU_E_TIMEOUT, "radix sort look-back wait gave up");
        c->bvh_valid = true;
        c->shapes_exported = false;
        st = prepare_bvh_trace(c);
        if (st) return st;
        CK(cudaStreamSynchronize(c->stream));
        c->accel_built = PTGPU_ACCEL_BVH;
        return PTGPU_OK;
    }
    // KD tree with the reference topology (on the GPU unless asked for the
    // host build), device traversal
    auto t0 = std::chrono::steady_clock::now();
    if (flags & PTGPU_FLAG_KD_HOST) {
        int st = ensure_host_shapes(c);
        if (st) return st;
        st = kd_build(c->h_shapes.data(), c->n, c->kd);
        if (st) return fail(st, "kd build failed");
    } else {
        if (!c->kd_scratch) c->kd_scratch = kd_scratch_create();
        CK(kd_build_gpu(c->d_verts.as<float>(), c->d_type.as<uint8_t>(), c->n, c->kd, *c->kd_scratch,
                        c->stream));
    }
    int st;
    if (c->host_shapes)
        for (uint32_t i = 0; i < c->n; ++i) { c->h_shapes[i].index = (int32_t)i; c->h_shapes[i].morton_code = 0; }
    c->kd_indexed = true;
    std::vector<float> nodes;
    float root_box[6];
    kd_trace_nodes(c->kd, nodes, &c->root_first, &c->root_count, root_box);
    const size_t nk = c->kd.kn.size();
    CK(c->d_nodes.ensure(nodes.size() * sizeof(float) + 64));
    CK(c->d_prims.ensure((nk ? nk : 1) * 3 * sizeof(float4)));
    CK(c->d_prim_id.ensure((nk ? nk : 1) * 4));
    CK(c->d_root_box.ensure(6 * sizeof(float)));
    if (!nodes.empty())
        CK(cudaMemcpyAsync(c->d_nodes.p, nodes.data(), nodes.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    if (nk)
        CK(cudaMemcpyAsync(c->d_prim_id.p, c->kd.kn.data(), nk * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_root_box.p, root_box, sizeof(root_box), cudaMemcpyHostToDevice, c->stream));
    CK(launch_gather_prims(c->d_prim_id.as<int32_t>(), (int)nk, c->d_prims0.as<float4>(),
                           c->d_prims.as<float4>(), c->stream));
    c->n_internal = (int)(nodes.size() / 16);
    st = prepare_wide(c);
    if (st) return st;
    CK(cudaStreamSynchronize(c->stream));
    c->last_build_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    c->kd_valid = true;
    c->accel_built = PTGPU_ACCEL_KDTREE;
    return PTGPU_OK;
}

static_assert(PTGPU_WAIT_LIMIT_DEFAULT == kDefaultWaitLimit, "header and build agree on the default");

int ptgpu_set_wait_limit(ptgpu_ctx *c, uint32_t polls) {
    if (!c) return fail(PTGPU_E_INVAL, "null context");
    c->wait_limit = polls;
    return PTGPU_OK;
}

int ptgpu_last_build_ms(ptgpu_ctx *c, float *ms) {
    if (!c || !ms) return fail(PTGPU_E_INVAL, "null argument");
    *ms = c->last_build_ms;
    return PTGPU_OK;
}

int ptgpu_get_bvh(ptgpu_ctx *c, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl) {
    if (!c || !btl || (!btn && c->n > 1)) return fail(PTGPU_E_INVAL, "null argument");
    if (!c->bvh_valid) return fail(PTGPU_E_STATE, "no BVH has been built");
    cudaSetDevice(c->device);
    if (c->n > 1)
        CK(cudaMemcpyAsync(btn, c->d_btn.p, (size_t)(c->n - 1) * sizeof(ptgpu_bvh_node), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(btl, c->d_btl.p, (size_t)c->n * sizeof(ptgpu_bvh_node), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PTGPU_OK;
}

int ptgpu_set_bvh(ptgpu_ctx *c, const ptgpu_bvh_node *btn, const ptgpu_bvh_node *btl, uint32_t n) {
    if (!c || !btl || (!btn && n > 1)) return fail(PTGPU_E_INVAL, "null argument");
    if (n != c->n) return fail(PTGPU_E_INVAL, "node count does not match the shape count");
    for (uint32_t k = 0; k < n; ++k)
        if (btl[k].nShape < 0 || (uint32_t)btl[k].nShape >= n) return fail(PTGPU_E_INVAL, "leaf shape out of range");
    for (uint32_t i = 0; i + 1 < n; ++i) {
        const ptgpu_bvh_node &d = btn[i];
        bool ll = d.nLeft == d.min, rl = d.nRight == d.max;
        if (d.nLeft < 0 || d.nRight < 0 || (uint32_t)d.nLeft >= (ll ? n : n - 1) ||
            (uint32_t)d.nRight >= (rl ? n : n - 1))
            return fail(PTGPU_E_INVAL, "child index out of range at node " + std::to_string(i));
    }
    cudaSetDevice(c->device);
    int st = ensure_bvh_buffers(c);
    if (st) return st;
    if (n > 1) CK(cudaMemcpyAsync(c->d_btn.p, btn, (size_t)(n - 1) * sizeof(ptgpu_bvh_node), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_btl.p, btl, (size_t)n * sizeof(ptgpu_bvh_node), cudaMemcpyHostToDevice, c->stream));
    c->bvh_valid = true;
    c->shapes_exported = true;   // shapes keep what the caller set
    st = prepare_bvh_trace(c);
    if (st) return st;
    CK(cudaStreamSynchronize(c->stream));
    c->accel_built = PTGPU_ACCEL_BVH;
    c->current_sample = 0;
    return PTGPU_OK;
}

int ptgpu_get_kdtree(ptgpu_ctx *c, ptgpu_kd_node *kng, int32_t *kng_cnt, int32_t *kn, int32_t *kn_cnt) {
    if (!c || !kng_cnt || !kn_cnt) return fail(PTGPU_E_INVAL, "null argument");
    if (!c->kd_valid) return fail(PTGPU_E_STATE, "no KD tree has been built");
    int64_t size;
    int st = kd_heap_size(c->kd, &size);
    *kn_cnt = c->kd.szbuf;
    if (size < 0 || size > INT32_MAX) { *kng_cnt = -1; return fail(PTGPU_E_RANGE, "KD heap too large"); }
    if (!kng || !kn) {          // size query
        *kng_cnt = (int32_t)size;
        return st == PTGPU_OK ? PTGPU_OK : fail(st, "KD tree does not fit the int16 layout");
    }
    if (*kng_cnt < size) return fail(PTGPU_E_INVAL, "kng buffer too small");
    *kng_cnt = (int32_t)size;
    st = kd_export_heap(c->kd, kng, size, kn);
    if (st) return fail(st, "KD tree does not fit the int16 layout");
    return PTGPU_OK;
}

int ptgpu_get_kdtree_wide(ptgpu_ctx *c, ptgpu_kd_node_wide *nodes, int32_t *node_cnt, int32_t *kn,
                          int32_t *kn_cnt) {
    if (!c || !node_cnt || !kn_cnt) return fail(PTGPU_E_INVAL, "null argument");
    if (!c->kd_valid) return fail(PTGPU_E_STATE, "no KD tree has been built");
    const int32_t cnt = c->kd.node_count();
    const int32_t kcnt = (int32_t)c->kd.kn.size();
    if (!nodes || !kn) {          // size query
        *node_cnt = cnt;
        *kn_cnt = kcnt;
        return PTGPU_OK;
    }
    if (*node_cnt < cnt || *kn_cnt < kcnt) return fail(PTGPU_E_INVAL, "node or kn buffer too small");
    kd_export_wide(c->kd, nodes);
    if (kcnt) std::memcpy(kn, c->kd.kn.data(), sizeof(int32_t) * (size_t)kcnt);
    *node_cnt = cnt;
    *kn_cnt = kcnt;
    return PTGPU_OK;
}

int ptgpu_encode_image(ptgpu_ctx *c, int32_t format, void *buf, uint64_t *size) {
    if (!c || !size) return fail(PTGPU_E_INVAL, "null argument");
    if (format != PTGPU_IMAGE_PPM && format != PTGPU_IMAGE_PFM) return fail(PTGPU_E_INVAL, "unknown image format");
    if (c->current_sample <= 0) return fail(PTGPU_E_STATE, "no frame has been drawn");
    cudaSetDevice(c->device);
    char header[80];
    int hl;
    uint64_t body;
    if (format == PTGPU_IMAGE_PPM) {
        hl = std::snprintf(header, sizeof(header), "P3\n%d %d\n%d\n", c->w, c->h, 255);
        CK(c->d_rowoff.ensure(((size_t)c->h + 1) * sizeof(uint64_t)));
        CK(launch_ppm_length(c->d_pixels.as<uint32_t>(), c->w, c->h, c->d_rowoff.as<uint64_t>(), c->stream));
        CK(cudaMemcpyAsync(&body, c->d_rowoff.as<uint64_t>() + c->h, sizeof(body), cudaMemcpyDeviceToHost,
                           c->stream));
        CK(cudaStreamSynchronize(c->stream));
    } else {
        hl = std::snprintf(header, sizeof(header), "PF\n%d %d\n-1.0\n", c->w, c->h);
        body = (uint64_t)c->w * c->h * 3 * sizeof(float);
    }
    const uint64_t need = (uint64_t)hl + body;
    if (!buf) { *size = need; return PTGPU_OK; }
    if (*size < need) { *size = need; return fail(PTGPU_E_INVAL, "image buffer too small"); }
    std::memcpy(buf, header, (size_t)hl);
    CK(c->d_img.ensure(body ? body : 1));
    if (format == PTGPU_IMAGE_PPM)
        CK(launch_ppm_write(c->d_pixels.as<uint32_t>(), c->w, c->h, c->d_rowoff.as<uint64_t>(), c->d_img.as<char>(),
                            c->stream));
    else
        CK(launch_pfm(c->d_colors.as<ptgpu_vec>(), c->w, c->h, c->d_img.as<float>(), c->sm_count, c->stream));
    CK(cudaMemcpyAsync(static_cast<char *>(buf) + hl, c->d_img.p, body, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *size = need;
    return PTGPU_OK;
}

int ptgpu_write_image(ptgpu_ctx *c, const char *path, int32_t format) {
    if (!c || !path) return fail(PTGPU_E_INVAL, "null argument");
    uint64_t size = 0;
    int st = ptgpu_encode_image(c, format, nullptr, &size);
    if (st) return st;
    std::vector<char> bytes;
    try {
        bytes.resize(size);
    } catch (const std::bad_alloc &) {
        return fail(PTGPU_E_OOM, "out of host memory for the image");
    }
    st = ptgpu_encode_image(c, format, bytes.data(), &size);
    if (st) return st;
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(PTGPU_E_IO, std::string("cannot open image file: ") + path);
    const size_t wrote = std::fwrite(bytes.data(), 1, bytes.size(), f);
    const bool ok = std::fclose(f) == 0 && wrote == bytes.size();
    return ok ? PTGPU_OK : fail(PTGPU_E_IO, std::string("cannot write image file: ") + path);
}

int ptgpu_set_seeds(ptgpu_ctx *c, const uint32_t *seeds) {
    if (!c || !seeds) return fail(PTGPU_E_INVAL, "null argument");
    cudaSetDevice(c->device);
    CK(cudaMemcpyAsync(c->d_seeds.p, seeds, (size_t)c->w * c->h * 2 * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PTGPU_OK;
}

int ptgpu_get_seeds(ptgpu_ctx *c, uint32_t *seeds) {
    if (!c || !seeds) return fail(PTGPU_E_INVAL, "null argument");
    cudaSetDevice(c->device);
    CK(cudaMemcpyAsync(seeds, c->d_seeds.p, (size_t)c->w * c->h * 2 * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PTGPU_OK;
}

int ptgpu_reset_accumulation(ptgpu_ctx *c) {
    if (!c) return fail(PTGPU_E_INVAL, "null context");
    c->current_sample = 0;
    return PTGPU_OK;
}

int ptgpu_get_current_sample(ptgpu_ctx *c, int32_t *cs) {
    if (!c || !cs) return fail(PTGPU_E_INVAL, "null argument");
    *cs = c->current_sample;
    return PTGPU_OK;
}

static int enqueue_render(ptgpu_ctx *c, uint32_t passes, unsigned long long *stats = nullptr) {
    if (c->accel_built < 0) return fail(PTGPU_E_STATE, "build an acceleration structure first");
    if (!c->cam_set) return fail(PTGPU_E_STATE, "set a camera first");
    if (passes == 0) return PTGPU_OK;
    RenderArgs a;
    std::memset(&a, 0, sizeof(a));
    a.tv = make_view(c);
    a.mats = c->d_mats.as<Material>();
    a.prims0 = c->d_prims0.as<float4>();
    a.lights = c->d_lights.as<LightRec>();
    a.n_lights = c->n_lights;
    a.cam = c->cam;
    a.width = c->w;
    a.height = c->h;
    a.start_sample = c->current_sample;
    a.passes = (int32_t)passes;
    a.max_depth = c->max_depth;
    a.rtl = c->rtl;
    a.rr_depth = c->rr_depth;
    a.colors = c->d_colors.as<ptgpu_vec>();
    a.pixels = c->d_pixels.as<uint32_t>();
    a.seeds = c->d_seeds.as<uint32_t>();
    a.stats = stats;
    a.pixel_counter = c->d_pixctr.as<unsigned int>();
    a.max_ctas = 0;
    if (!stats && (c->flags & PTGPU_FLAG_WAVEFRONT) && c->n_lights <= kWfMaxLights) {
        // path slots: all pixels at once unless that needs more than 2 GB
        const int npx = c->w * c->h;
        int paths = npx;
        while (paths > 4096 && wf_carve_bytes(paths, c->n_lights) > (size_t(2) << 30)) paths = (paths + 1) / 2;
        CK(c->d_wf.ensure(wf_carve_bytes(paths, c->n_lights)));
        WfArgs w;
        std::memset(&w, 0, sizeof(w));
        w.r = a;
        w.paths = paths;
        wf_carve(w, c->d_wf.p, paths, c->n_lights);
        const int grid = c->sm_count * 12;
        CK(launch_wavefront(w, (int)passes * (c->max_depth + 1), grid, c->stream));
    } else {
        // pixels handed out in decreasing work of the previous frame, so the
        // frame ends on short pixel chains (first frame: row order)
        const int npx = c->w * c->h;
        CK(c->d_cost.ensure((size_t)npx * sizeof(uint32_t)));
        CK(c->d_order.ensure((size_t)npx * sizeof(int32_t)));
        CK(c->d_order_scr.ensure(2 * kOrderScratchWords * sizeof(uint32_t)));
        const bool reorder = !(c->flags & PTGPU_FLAG_ROW_ORDER);
        a.order = reorder && c->order_valid ? c->d_order.as<int32_t>() : nullptr;
        a.cost = reorder ? c->d_cost.as<uint32_t>() : nullptr;
        CK(launch_render(a, c->block, c->stream));
        if (reorder) {
            CK(launch_pixel_order(c->d_cost.as<uint32_t>(), c->d_order.as<int32_t>(),
                                  c->d_order_scr.as<uint32_t>(), npx, c->stream));
            c->order_valid = true;
        }
    }
    c->current_sample += (int)passes;
    return PTGPU_OK;
}

static int check_err_flags(ptgpu_ctx *c) {
    int32_t flags = 0;
    CK(cudaMemcpyAsync(&flags, c->d_err.p, 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (flags & 1) {
        cudaMemsetAsync(c->d_err.p, 0, 4, c->stream);
        return fail(PTGPU_E_RANGE, "traversal stack overflow (tree deeper than 64 levels)");
    }
    return PTGPU_OK;
}

int ptgpu_draw_frame(ptgpu_ctx *c, uint32_t passes, const uint32_t **pixels_out) {
    if (!c) return fail(PTGPU_E_INVAL, "null context");
    cudaSetDevice(c->device);
    int st = enqueue_render(c, passes);
    if (st) return st;
    CK(cudaMemcpyAsync(c->h_pixels, c->d_pixels.p, (size_t)c->w * c->h * 4, cudaMemcpyDeviceToHost, c->stream));
    st = check_err_flags(c);
    if (st) return st;
    if (pixels_out) *pixels_out = c->h_pixels;
    return PTGPU_OK;
}

int ptgpu_render_async(ptgpu_ctx *c, uint32_t passes) {
    if (!c) return fail(PTGPU_E_INVAL, "null context");
    cudaSetDevice(c->device);
    return enqueue_render(c, passes);
}

int ptgpu_render_stats(ptgpu_ctx *c, uint32_t passes, uint64_t *stats) {
    if (!c || !stats) return fail(PTGPU_E_INVAL, "null argument");
    cudaSetDevice(c->device);
    unsigned long long *d = nullptr;
    CK(cudaMalloc(&d, 6 * sizeof(unsigned long long)));
    cudaError_t e = cudaMemsetAsync(d, 0, 6 * sizeof(unsigned long long), c->stream);
    int st = e == cudaSuccess ? enqueue_render(c, passes, d) : cuda_fail(e, "memset stats");
    if (st == PTGPU_OK) {
        e = cudaMemcpyAsync(stats, d, 6 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) st = cuda_fail(e, "read stats");
    }
    cudaFree(d);
    return st;
}

int ptgpu_synchronize(ptgpu_ctx *c) {
    if (!c) return fail(PTGPU_E_INVAL, "null context");
    cudaSetDevice(c->device);
    CK(cudaStreamSynchronize(c->stream));
    return check_err_flags(c);
}

int ptgpu_get_colors(ptgpu_ctx *c, ptgpu_vec *colors) {
    if (!c || !colors) return fail(PTGPU_E_INVAL, "null argument");
    cudaSetDevice(c->device);
    CK(cudaMemcpyAsync(colors, c->d_colors.p, (size_t)c->w * c->h * sizeof(ptgpu_vec), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PTGPU_OK;
}

int ptgpu_get_pixels(ptgpu_ctx *c, uint32_t *pixels) {
    if (!c || !pixels) return fail(PTGPU_E_INVAL, "null argument");
    cudaSetDevice(c->device);
    CK(cudaMemcpyAsync(pixels, c->d_pixels.p, (size_t)c->w * c->h * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PTGPU_OK;
}

int ptgpu_trace_closest_device(ptgpu_ctx *c, const ptgpu_ray *d_rays, uint32_t n, float *d_t,
                               uint32_t *d_id, int32_t *d_hit) {
    if (!c || (n && (!d_rays || !d_t || !d_id || !d_hit))) return fail(PTGPU_E_INVAL, "null argument");
    if (c->accel_built < 0) return fail(PTGPU_E_STATE, "build an acceleration structure first");
    cudaSetDevice(c->device);
    CK(launch_trace_closest(make_view(c), d_rays, (int)n, d_t, d_id, d_hit, c->stream,
                            c->d_pixctr.as<unsigned int>() + 1));
    return PTGPU_OK;
}

int ptgpu_trace_closest_stats(ptgpu_ctx *c, const ptgpu_ray *d_rays, uint32_t n, float *d_t,
                              uint32_t *d_id, int32_t *d_hit, uint64_t *stats) {
    if (!c || !stats || (n && (!d_rays || !d_t || !d_id || !d_hit))) return fail(PTGPU_E_INVAL, "null argument");
    if (c->accel_built < 0) return fail(PTGPU_E_STATE, "build an acceleration structure first");
    cudaSetDevice(c->device);
    unsigned long long *d = nullptr;
    CK(cudaMalloc(&d, 2 * sizeof(unsigned long long)));
    cudaError_t e = cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), c->stream);
    if (e == cudaSuccess)
        e = launch_trace_closest(make_view(c), d_rays, (int)n, d_t, d_id, d_hit, c->stream,
                                 c->d_pixctr.as<unsigned int>() + 1, d);
    if (e == cudaSuccess) e = cudaMemcpyAsync(stats, d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "closest-hit counters");
    return PTGPU_OK;
}

int ptgpu_trace_closest(ptgpu_ctx *c, const ptgpu_ray *rays, uint32_t n, float *t, uint32_t *id,
                        int32_t *hit) {
    if (!c || (n && (!rays || !t || !id || !hit))) return fail(PTGPU_E_INVAL, "null argument");
    if (c->accel_built < 0) return fail(PTGPU_E_STATE, "build an acceleration structure first");
    if (n == 0) return PTGPU_OK;
    cudaSetDevice(c->device);
    CK(c->d_rays.ensure((size_t)n * sizeof(ptgpu_ray)));
    CK(c->d_t.ensure((size_t)n * 4));
    CK(c->d_id.ensure((size_t)n * 4));
    CK(c->d_hit.ensure((size_t)n * 4));
    CK(cudaMemcpyAsync(c->d_rays.p, rays, (size_t)n * sizeof(ptgpu_ray), cudaMemcpyHostToDevice, c->stream));
    CK(launch_trace_closest(make_view(c), c->d_rays.as<ptgpu_ray>(), (int)n, c->d_t.as<float>(),
                            c->d_id.as<uint32_t>(), c->d_hit.as<int32_t>(), c->stream,
                            c->d_pixctr.as<unsigned int>() + 1));
    CK(cudaMemcpyAsync(t, c->d_t.p, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(id, c->d_id.p, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(hit, c->d_hit.p, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
    return check_err_flags(c);
}

}  // extern "C"

// C entry points: no C++ exception crosses the C ABI
int ptgpu_set_shapes(ptgpu_ctx *c, const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt) {
    try {
        return ptgpu_set_shapes_body(c, shapes, n, light_cnt);
    } catch (const std::bad_alloc &) {
        return fail(PTGPU_E_OOM, "out of host memory");
    } catch (const std::exception &e) {
        return fail(PTGPU_E_INVAL, std::string("unexpected error: ") + e.what());
    }
}

int ptgpu_get_shapes(ptgpu_ctx *c, ptgpu_shape *out, uint32_t n) {
    try {
        return ptgpu_get_shapes_body(c, out, n);
    } catch (const std::bad_alloc &) {
        return fail(PTGPU_E_OOM, "out of host memory");
    } catch (const std::exception &e) {
        return fail(PTGPU_E_INVAL, std::string("unexpected error: ") + e.what());
    }
}

int ptgpu_read_scene(ptgpu_ctx *c, const char *path, int32_t *walllight) {
    try {
        return ptgpu_read_scene_body(c, path, walllight);
    } catch (const std::bad_alloc &) {
        return fail(PTGPU_E_OOM, "out of host memory");
    } catch (const std::exception &e) {
        return fail(PTGPU_E_INVAL, std::string("unexpected error: ") + e.what());
    }
}

int ptgpu_stream_scene(ptgpu_ctx *c, const char *path, int32_t *walllight) {
    try {
        return ptgpu_stream_scene_body(c, path, walllight);
    } catch (const std::bad_alloc &) {
        return fail(PTGPU_E_OOM, "out of host memory");
    } catch (const std::exception &e) {
        return fail(PTGPU_E_INVAL, std::string("unexpected error: ") + e.what());
    }
}

int ptgpu_build(ptgpu_ctx *c, int32_t accel, uint32_t flags) {
    try {
        return ptgpu_build_body(c, accel, flags);
    } catch (const std::bad_alloc &) {
        return fail(PTGPU_E_OOM, "out of host memory");
    } catch (const std::exception &e) {
        return fail(PTGPU_E_INVAL, std::string("unexpected error: ") + e.what());
    }
}
