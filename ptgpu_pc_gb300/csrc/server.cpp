// server.cpp -- render serving with continuous batching (ptgpu_server_*).
//
// One worker thread owns the device state.  Resident scenes live in shared
// "shape-slot" arenas: a scene of n shapes holds the slot range [base,
// base+n) of the primitive, shape-id, material and shape-order arrays and
// [base, base+n-1) of the node array, so the batched render kernel reaches
// every resident scene through one set of arrays and a per-request record
// (root, first shape, lights, camera, size, passes).  Accumulation buffers
// (colours, pixels, seeds) of admitted requests live in a pixel arena.  Both
// arenas grow by doubling up to the byte budget; a request is admitted when
// its scene is resident or can be built, and its pixels fit, possibly after
// evicting scenes no admitted request uses (least recently used first).
//
// Each step renders up to `quantum` passes of the oldest admitted requests
// whose pixels fit one filling of the GPU (or of every admitted request, with
// PTGPU_SERVER_ALL_ACTIVE; at most 256 per launch) starting at the request's
// sample count, so a request
// refines progressively and new requests join at step boundaries.  The
// running mean and the seeds are stored and reloaded between steps exactly
// as the kernel keeps them in registers within one launch, so a request's
// result does not depend on how its passes fall into steps.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "devbuf.h"
#include "host.h"
#include "ingest.h"
#include "lbvh.h"
#include "range_alloc.h"
#include "step_policy.h"

using namespace ptgpu;

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point t0, Clock::time_point t1) {
    return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

// A device array that grows by copying its old contents (indices stay valid).
struct Arena {
    DevBuf buf;
    size_t elem = 1;
    cudaError_t grow(int64_t old_n, int64_t new_n, cudaStream_t s) {
        DevBuf nb;
        cudaError_t e = nb.ensure((size_t)new_n * elem);
        if (e != cudaSuccess) return e;
        if (buf.p && old_n > 0) {
            e = cudaMemcpyAsync(nb.p, buf.p, (size_t)old_n * elem, cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) { nb.release(); return e; }
        }
        buf.release();
        buf = nb;
        nb.p = nullptr;
        return cudaSuccess;
    }
};

// bytes per shape slot: nodes 64, prims 48, prim_id 4, materials 32, shape-order prims 48
constexpr int64_t kSlotBytes = 64 + 48 + 4 + 32 + 48;
// bytes per pixel slot: colour 12, pixel 4, seeds 8
constexpr int64_t kPixBytes = 12 + 4 + 8;

struct SceneEntry {
    // fixed when the scene is added: shapes and light records in host memory,
    // or a scene file that each build reads again (no host copy is kept)
    std::vector<ptgpu_shape> shapes;
    std::string path;                    // scene file, when shapes is empty
    int64_t n_shapes = 0;
    int n_lights = 0;
    uint32_t light_cnt = 0;
    uint32_t build_flags = 0;
    std::vector<LightRec> lights;
    // the worker's
    std::atomic<bool> resident{false};
    int depth = 0;                       // deepest leaf of its tree
    int64_t base = 0, light_base = 0;
    float root_box[6] = {0, 0, 0, 0, 0, 0};
    int users = 0;                       // admitted requests using it
    std::list<int>::iterator lru;        // position in the LRU list when resident
};

struct Request {
    int64_t ticket = 0;
    ptgpu_request r{};
    Clock::time_point t_submit, t_admit, t_done;
    int64_t pix_base = 0;
    int done_passes = 0;
    int steps = 0;
    int built = 0;
    int status = PTGPU_OK;
    bool finished = false;
    std::atomic<bool> cancel{false};     // set by ptgpu_server_cancel, acted on by the worker
    std::vector<uint32_t> pixels;
    std::vector<ptgpu_vec> colors;
};

// A progressive-preview copy of a request's image, made by the worker
// between two steps (ptgpu_server_preview waits for it).
struct PreviewJob {
    std::shared_ptr<Request> q;
    uint32_t *pixels = nullptr;
    ptgpu_vec *colors = nullptr;
    int passes = 0;
    int status = PTGPU_OK;
    bool done = false;
};

int cuda_fail(cudaError_t e, const char *what) {
    const int code = (e == cudaErrorMemoryAllocation) ? PTGPU_E_OOM : PTGPU_E_DEVICE;
    return record_error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

struct ptgpu_server {
    int device = 0;
    int64_t budget = 0;
    int quantum = 4;
    bool fill_cap = true;      // false with PTGPU_SERVER_ALL_ACTIVE
    int rtl = 0;
    int sm_count = 1;
    cudaStream_t stream = nullptr;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    int64_t next_ticket = 1;
    std::deque<std::shared_ptr<Request>> pending;                 // arrival order
    std::deque<std::shared_ptr<PreviewJob>> previews;             // to serve between steps
    std::unordered_map<int64_t, std::shared_ptr<Request>> tickets;
    std::vector<std::unique_ptr<SceneEntry>> scenes;              // by id (the vector: mu)
    // worker-only state
    std::vector<std::shared_ptr<Request>> active;
    std::list<int> lru;                                           // front = least recent
    RangeAlloc shape_slots, pix_slots, light_slots;
    Arena nodes, prims, prim_id, mats, prims0, lights, colors, pixels, seeds;
    DevBuf d_recs, d_pix_start, d_pixctr, d_err, d_seg, d_depth;
    // single-scene build scratch
    DevBuf s_shapes, s_verts, s_type, s_aabbs, s_keys, s_keys_alt, s_keys_tmp, s_vals_alt,
        s_vals_tmp, s_sorted, s_status, s_state, s_bb, s_arr, s_btn, s_btl, s_tcount, s_tcost;
    IngestScratch ingest;                                         // scene files
    std::atomic<int> n_active{0};                                 // active.size() for readers
    // counters (guarded by mu)
    int64_t done_count = 0, builds = 0, evictions = 0, steps = 0;
    double samples_done = 0.0;
    int last_error = PTGPU_OK;
    // the worker's slot counts as of its last release or admission (mu)
    int64_t shape_slots_used = 0, pixel_slots_used = 0, light_slots_used = 0;

    int64_t bytes_in_use() const {
        return shape_slots.capacity * kSlotBytes + pix_slots.capacity * kPixBytes +
               light_slots.capacity * (int64_t)sizeof(LightRec);
    }
};

namespace {

SceneEntry &scene_of(ptgpu_server *s, int id) {
    std::lock_guard<std::mutex> lk(s->mu);
    return *s->scenes[id];
}

// Grows the shape arenas so that `need` contiguous slots fit (the free
// range at the end of the arena counts), within the budget.
int grow_shapes(ptgpu_server *s, int64_t need) {
    const int64_t cap = s->shape_slots.capacity;
    const int64_t min_cap = cap + need - s->shape_slots.free_tail();
    int64_t want = std::max<int64_t>(cap * 2, min_cap);
    want = std::max<int64_t>(want, 4096);
    const int64_t room = (s->budget - s->bytes_in_use()) / kSlotBytes + cap;
    if (want > room) want = room;
    if (want < min_cap) return PTGPU_E_OOM;
    Arena *as[] = {&s->nodes, &s->prims, &s->prim_id, &s->mats, &s->prims0};
    for (Arena *a : as) {
        cudaError_t e = a->grow(cap, want, s->stream);
        if (e != cudaSuccess) return cuda_fail(e, "shape arena");
    }
    s->shape_slots.grow(want);
    return PTGPU_OK;
}

int grow_pixels(ptgpu_server *s, int64_t need) {
    const int64_t cap = s->pix_slots.capacity;
    const int64_t min_cap = cap + need - s->pix_slots.free_tail();
    int64_t want = std::max<int64_t>(cap * 2, min_cap);
    want = std::max<int64_t>(want, 16384);
    const int64_t room = (s->budget - s->bytes_in_use()) / kPixBytes + cap;
    if (want > room) want = room;
    if (want < min_cap) return PTGPU_E_OOM;
    Arena *as[] = {&s->colors, &s->pixels, &s->seeds};
    for (Arena *a : as) {
        cudaError_t e = a->grow(cap, want, s->stream);
        if (e != cudaSuccess) return cuda_fail(e, "pixel arena");
    }
    s->pix_slots.grow(want);
    return PTGPU_OK;
}

int grow_lights(ptgpu_server *s, int64_t need) {
    const int64_t cap = s->light_slots.capacity;
    const int64_t min_cap = cap + need - s->light_slots.free_tail();
    int64_t want = std::max<int64_t>(std::max<int64_t>(cap * 2, min_cap), 256);
    const int64_t room = (s->budget - s->bytes_in_use()) / (int64_t)sizeof(LightRec) + cap;
    if (want > room) want = room;
    if (want < min_cap) return PTGPU_E_OOM;
    cudaError_t e = s->lights.grow(cap, want, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "light arena");
    s->light_slots.grow(want);
    return PTGPU_OK;
}

void evict(ptgpu_server *s, int id) {
    SceneEntry &sc = scene_of(s, id);
    s->shape_slots.release(sc.base, sc.n_shapes);
    if (sc.n_lights > 0) s->light_slots.release(sc.light_base, (int64_t)sc.n_lights);
    s->lru.erase(sc.lru);
    sc.resident = false;
    std::lock_guard<std::mutex> lk(s->mu);
    s->evictions++;
}

// Frees shape slots by evicting unused resident scenes, least recent first,
// until `n` contiguous slots can be had.  Returns false if it cannot.
bool alloc_shapes(ptgpu_server *s, int64_t n, int64_t *base) {
    for (;;) {
        if (s->shape_slots.alloc(n, base)) return true;
        if (grow_shapes(s, n) == PTGPU_OK && s->shape_slots.alloc(n, base)) return true;
        int victim = -1;
        for (int id : s->lru)
            if (scene_of(s, id).users == 0) { victim = id; break; }
        if (victim < 0) return false;
        evict(s, victim);
    }
}

// Pixel slots come from the pixel arena alone (evicting scenes frees shape
// slots, not budget: the arenas keep their size).
bool alloc_pixels(ptgpu_server *s, int64_t n, int64_t *base) {
    if (s->pix_slots.alloc(n, base)) return true;
    return grow_pixels(s, n) == PTGPU_OK && s->pix_slots.alloc(n, base);
}

#define SK(expr)                                                   \
    do {                                                           \
        cudaError_t e_ = (expr);                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);        \
    } while (0)

// Builds scene `id` into freshly allocated slots (single-scene build in the
// scratch buffers, then the traversal arrays written at the slot base).
int build_scene(ptgpu_server *s, int id) {
    SceneEntry &sc = scene_of(s, id);
    const int n = (int)sc.n_shapes;
    int64_t base = 0;
    if (!alloc_shapes(s, n, &base)) return record_error(PTGPU_E_OOM, "scene does not fit the budget");
    int64_t lbase = 0;
    // The slots go back to their arenas on every failure below (a device
    // error, a scene file that changed or vanished, a look-back timeout); only
    // a scene that became resident keeps them, until it is evicted.
    struct SlotGuard {
        ptgpu_server *s;
        int64_t base, n, lbase = 0, nl = 0;
        bool keep = false;
        ~SlotGuard() {
            if (keep) return;
            s->shape_slots.release(base, n);
            if (nl > 0) s->light_slots.release(lbase, nl);
        }
    } guard{s, base, (int64_t)n};
    if (sc.n_lights > 0) {
        if (!s->light_slots.alloc((int64_t)sc.n_lights, &lbase)) {
            if (grow_lights(s, (int64_t)sc.n_lights) != PTGPU_OK ||
                !s->light_slots.alloc((int64_t)sc.n_lights, &lbase))
                return record_error(PTGPU_E_OOM, "the scene's lights do not fit the budget");
        }
        guard.lbase = lbase;
        guard.nl = (int64_t)sc.n_lights;
        if (!sc.lights.empty())
            SK(cudaMemcpyAsync(s->lights.buf.as<LightRec>() + lbase, sc.lights.data(),
                               sc.lights.size() * sizeof(LightRec), cudaMemcpyHostToDevice, s->stream));
    }
    const size_t N = (size_t)n;
    SK(s->s_shapes.ensure(N * sizeof(ptgpu_shape)));
    SK(s->s_verts.ensure(N * 9 * sizeof(float)));
    SK(s->s_type.ensure(N));
    SK(s->s_aabbs.ensure(N * 2 * sizeof(float4)));
    SK(s->s_keys.ensure(N * 4));
    SK(s->s_keys_alt.ensure(N * 4));
    SK(s->s_keys_tmp.ensure(N * 4));
    SK(s->s_vals_alt.ensure(N * 4));
    SK(s->s_vals_tmp.ensure(N * 4));
    SK(s->s_sorted.ensure(N * 4));
    SK(s->s_status.ensure(sort_status_words(n) * 4));
    SK(s->s_state.ensure(sizeof(BuildState)));
    SK(s->s_bb.ensure(block_bound_count(n) * 6 * sizeof(float)));
    SK(s->s_arr.ensure(block_bound_count(n) * sizeof(uint32_t)));
    SK(s->s_btn.ensure((N - 1) * sizeof(ptgpu_bvh_node)));
    SK(s->s_btl.ensure(N * sizeof(ptgpu_bvh_node)));
    if (sc.path.empty()) {
        SK(cudaMemcpyAsync(s->s_shapes.p, sc.shapes.data(), N * sizeof(ptgpu_shape), cudaMemcpyHostToDevice,
                           s->stream));
    } else {   // a cold scene file: read again and expanded on the device
        CompactScene cs;
        std::string err;
        int st = read_scene_compact(sc.path.c_str(), 1, 1, cs, err);
        if (st != PTGPU_OK) return record_error(st, err);
        if (cs.walllight) add_wall_light(cs);
        if (cs.count() != sc.n_shapes || (int)compact_light_count(cs) != sc.n_lights)
            return record_error(PTGPU_E_IO, "scene file changed since it was added: " + sc.path);
        SK(ingest_compact(cs, s->s_shapes.as<ptgpu_shape>(), s->lights.buf.as<LightRec>() + lbase, s->ingest,
                          s->stream));
    }
    float4 *prims0 = s->prims0.buf.as<float4>() + 3 * base;
    SK(launch_unpack_shapes(s->s_shapes.as<ptgpu_shape>(), n, s->s_verts.as<float>(), s->s_type.as<uint8_t>(),
                            prims0, s->mats.buf.as<Material>() + base, s->stream));
    LbvhBuffers b;
    std::memset(&b, 0, sizeof(b));
    b.wait_limit = kDefaultWaitLimit;
    b.verts = s->s_verts.as<float>();
    b.type = s->s_type.as<uint8_t>();
    b.aabbs = s->s_aabbs.as<float4>();
    b.leaf_bounds = nullptr;                     // batched builds only
    b.keys = s->s_keys.as<uint32_t>();
    b.keys_alt = s->s_keys_alt.as<uint32_t>();
    b.keys_tmp = s->s_keys_tmp.as<uint32_t>();
    b.vals_alt = s->s_vals_alt.as<int32_t>();
    b.vals_tmp = s->s_vals_tmp.as<int32_t>();
    b.sorted = s->s_sorted.as<int32_t>();
    b.status = s->s_status.as<uint32_t>();
    b.state = s->s_state.as<BuildState>();
    b.block_bounds = s->s_bb.as<float>();
    b.arrivals = s->s_arr.as<uint32_t>();
    b.btn = s->s_btn.as<ptgpu_bvh_node>();
    b.btl = s->s_btl.as<ptgpu_bvh_node>();
    SK(launch_lbvh_build(b, n, 0, s->sm_count, s->stream));
    if (sc.build_flags & PTGPU_FLAG_TREELET) {
        const int sweeps = ((sc.build_flags >> 8) & 0xF) ? (int)((sc.build_flags >> 8) & 0xF) : 1;
        SK(s->s_tcount.ensure(N * sizeof(int)));
        SK(s->s_tcost.ensure(N * sizeof(float)));
        SK(launch_treelet(b.btn, b.btl, n, s->s_tcount.as<int>(), s->s_tcost.as<float>(), sweeps, s->stream));
    }
    SK(launch_abi_to_trace(b.btn, b.btl, n, prims0, s->nodes.buf.as<float4>() + 4 * base,
                           s->prims.buf.as<float4>() + 3 * base, s->prim_id.buf.as<int32_t>() + base,
                           s->stream, (int)base, (int)base));
    const int32_t seg[2] = {0, n};
    SK(s->d_seg.ensure(sizeof(seg)));
    SK(cudaMemcpyAsync(s->d_seg.p, seg, sizeof(seg), cudaMemcpyHostToDevice, s->stream));
    SK(launch_tree_depth(b.btn, b.btl, s->d_seg.as<int32_t>(), 1, n, s->d_depth.as<int>(), s->stream));
    ptgpu_bound rb;
    uint32_t err_word = 0;
    int depth = 0;
    SK(cudaMemcpyAsync(&depth, s->d_depth.p, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    SK(cudaMemcpyAsync(&rb, &b.btn[0].bound, sizeof(rb), cudaMemcpyDeviceToHost, s->stream));
    SK(cudaMemcpyAsync(&err_word, &b.state->error, sizeof(err_word), cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    if (err_word) return record_error(PTGPU_E_TIMEOUT, "radix sort look-back wait gave up");
    sc.root_box[0] = rb.min_x; sc.root_box[1] = rb.max_x; sc.root_box[2] = rb.min_y;
    sc.root_box[3] = rb.max_y; sc.root_box[4] = rb.min_z; sc.root_box[5] = rb.max_z;
    sc.base = base;
    sc.light_base = lbase;
    sc.depth = depth;
    sc.resident = true;
    guard.keep = true;
    s->lru.push_back(id);
    sc.lru = std::prev(s->lru.end());
    std::lock_guard<std::mutex> lk(s->mu);
    s->builds++;
    return PTGPU_OK;
}

// (worker thread, mu held) the slot counts that ptgpu_server_info_get reports
void publish_usage_locked(ptgpu_server *s) {
    s->shape_slots_used = s->shape_slots.used;
    s->pixel_slots_used = s->pix_slots.used;
    s->light_slots_used = s->light_slots.used;
}

void finish(ptgpu_server *s, const std::shared_ptr<Request> &r, int status) {
    std::lock_guard<std::mutex> lk(s->mu);
    publish_usage_locked(s);
    r->status = status;
    r->finished = true;
    r->t_done = Clock::now();
    if (status == PTGPU_OK) {
        s->done_count++;
        s->samples_done += (double)r->r.width * r->r.height * r->r.spp;
    }
    s->cv_done.notify_all();
}

// Cancelled requests that have not been admitted leave the queue (only the
// worker removes requests from it, so no admission is in flight here).
void drop_cancelled_pending(ptgpu_server *s) {
    std::vector<std::shared_ptr<Request>> gone;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto it = s->pending.begin(); it != s->pending.end();) {
            if ((*it)->cancel) { gone.push_back(*it); it = s->pending.erase(it); }
            else ++it;
        }
    }
    for (auto &q : gone) finish(s, q, PTGPU_E_CANCELED);
}

// Active requests that were cancelled give their pixel slots back and end
// before the next step.
void drop_cancelled_active(ptgpu_server *s) {
    std::vector<std::shared_ptr<Request>> keep;
    for (auto &q : s->active) {
        if (!q->cancel) { keep.push_back(q); continue; }
        s->pix_slots.release(q->pix_base, (int64_t)q->r.width * q->r.height);
        scene_of(s, q->r.scene).users--;
        finish(s, q, PTGPU_E_CANCELED);
    }
    s->active.swap(keep);
    s->n_active = (int)s->active.size();
}

// Serves the queued preview copies: an active request's image as of its
// last finished step, a finished one's final image.
void serve_previews(ptgpu_server *s) {
    std::deque<std::shared_ptr<PreviewJob>> jobs;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        jobs.swap(s->previews);
    }
    for (auto &j : jobs) {
        Request &q = *j->q;
        const int64_t px = (int64_t)q.r.width * q.r.height;
        bool active = false;
        for (auto &a : s->active) active = active || a.get() == &q;
        bool fin;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            fin = q.finished;
        }
        if (active) {
            cudaError_t e = cudaSuccess;
            if (j->pixels)
                e = cudaMemcpyAsync(j->pixels, s->pixels.buf.as<uint32_t>() + q.pix_base, px * sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess && j->colors)
                e = cudaMemcpyAsync(j->colors, s->colors.buf.as<ptgpu_vec>() + q.pix_base,
                                    px * sizeof(ptgpu_vec), cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            j->passes = q.done_passes;
            j->status = e == cudaSuccess ? PTGPU_OK : cuda_fail(e, "preview copy");
        } else if (fin && q.status == PTGPU_OK) {
            if (j->pixels) std::memcpy(j->pixels, q.pixels.data(), px * sizeof(uint32_t));
            if (j->colors) std::memcpy(j->colors, q.colors.data(), px * sizeof(ptgpu_vec));
            j->passes = q.r.spp;
        } else if (fin) {
            j->status = q.status;
        } else {
            j->status = PTGPU_E_STATE;     // not admitted yet: no pass rendered
        }
        std::lock_guard<std::mutex> lk(s->mu);
        j->done = true;
        s->cv_done.notify_all();
    }
}

// Admits pending requests in arrival order while they fit.
void admit(ptgpu_server *s) {
    drop_cancelled_pending(s);
    for (;;) {
        std::shared_ptr<Request> r;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            publish_usage_locked(s);
            if (s->pending.empty() || s->active.size() >= (size_t)kMaxSegments) return;
            r = s->pending.front();
        }
        SceneEntry &sc = scene_of(s, r->r.scene);
        const int64_t px = (int64_t)r->r.width * r->r.height;
        const int64_t need = sc.n_shapes * kSlotBytes + px * kPixBytes;
        if (need > s->budget) {
            { std::lock_guard<std::mutex> lk(s->mu); s->pending.pop_front(); }
            record_error(PTGPU_E_RANGE, "request can never fit the budget");
            finish(s, r, PTGPU_E_RANGE);
            continue;
        }
        sc.users++;                        // pin the scene while its pixels are placed
        int built = 0;
        if (!sc.resident) {
            const int st = build_scene(s, r->r.scene);
            if (st != PTGPU_OK) {
                sc.users--;
                if (st == PTGPU_E_OOM && !s->active.empty()) return;   // wait for room
                { std::lock_guard<std::mutex> lk(s->mu); s->pending.pop_front(); }
                finish(s, r, st);
                continue;
            }
            built = 1;
        }
        int64_t pb = 0;
        if (!alloc_pixels(s, px, &pb)) {
            sc.users--;
            if (!s->active.empty()) return;   // wait until running requests free room
            { std::lock_guard<std::mutex> lk(s->mu); s->pending.pop_front(); }
            record_error(PTGPU_E_OOM, "request pixels do not fit the budget");
            finish(s, r, PTGPU_E_OOM);
            continue;
        }
        s->lru.splice(s->lru.end(), s->lru, sc.lru);   // most recently used
        std::vector<uint32_t> seeds(2 * (size_t)px);
        make_seeds(r->r.seed, seeds.data(), (uint32_t)seeds.size());
        cudaError_t e = cudaMemcpyAsync(s->seeds.buf.as<uint32_t>() + 2 * pb, seeds.data(),
                                        seeds.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->pending.pop_front();
        }
        if (e != cudaSuccess) {
            s->pix_slots.release(pb, px);
            sc.users--;
            finish(s, r, cuda_fail(e, "seed upload"));
            continue;
        }
        r->pix_base = pb;
        r->built = built;
        r->t_admit = Clock::now();
        s->active.push_back(r);
        s->n_active = (int)s->active.size();
    }
}

// One step: up to `quantum` passes of the oldest admitted requests whose
// pixels fit one filling of the GPU (with PTGPU_SERVER_ALL_ACTIVE: of every
// admitted request), one launch.
int step(ptgpu_server *s) {
    drop_cancelled_active(s);
    const int A = (int)s->active.size();
    if (A == 0) return PTGPU_OK;
    int depth = 0;
    for (int k = 0; k < A; ++k) depth = std::max(depth, scene_of(s, s->active[k]->r.scene).depth);
    // a binary traversal pushes at most two words per level
    const int stack = render_stack_for_depth(depth);
    const int grid = render_batch_grid(128, stack, 0);
    // the requests of this step, oldest first (active is in admission order)
    std::vector<int64_t> px(A);
    for (int k = 0; k < A; ++k) px[k] = (int64_t)s->active[k]->r.width * s->active[k]->r.height;
    const std::vector<int> sel = step_selection(px, s->fill_cap, (int64_t)grid * 128 * 4);
    const int S = (int)sel.size();
    std::vector<BatchScene> recs(S);
    std::vector<int64_t> start(S + 1, 0);
    for (int k = 0; k < S; ++k) {
        const Request &q = *s->active[sel[k]];
        const SceneEntry &sc = scene_of(s, q.r.scene);
        BatchScene &r = recs[k];
        std::memset(&r, 0, sizeof(r));
        r.cam = q.r.camera;
        r.width = q.r.width;
        r.height = q.r.height;
        r.passes = std::min(s->quantum, q.r.spp - q.done_passes);
        r.max_depth = q.r.max_depth ? q.r.max_depth : PTGPU_MAX_DEPTH;
        r.start_sample = q.done_passes;
        r.root = (int32_t)sc.base;
        r.n_shapes = (int32_t)sc.n_shapes;
        r.skip = (int32_t)(sc.base + sc.n_shapes - 1);
        r.shape0 = (int32_t)sc.base;
        r.light_first = (int32_t)sc.light_base;
        r.n_lights = (int32_t)sc.n_lights;
        r.pix_off = q.pix_base;
        std::memcpy(r.root_box, sc.root_box, sizeof(r.root_box));
        start[k + 1] = start[k] + (int64_t)q.r.width * q.r.height;
    }
    SK(s->d_recs.ensure(S * sizeof(BatchScene)));
    SK(s->d_pix_start.ensure((S + 1) * sizeof(int64_t)));
    SK(cudaMemcpyAsync(s->d_recs.p, recs.data(), S * sizeof(BatchScene), cudaMemcpyHostToDevice, s->stream));
    SK(cudaMemcpyAsync(s->d_pix_start.p, start.data(), (S + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                       s->stream));
    RenderArgs a;
    std::memset(&a, 0, sizeof(a));
    a.tv.nodes = s->nodes.buf.as<float4>();
    a.tv.prims = s->prims.buf.as<float4>();
    a.tv.prim_id = s->prim_id.buf.as<int32_t>();
    a.tv.accel = PTGPU_ACCEL_BVH;
    a.tv.error_flags = s->d_err.as<int32_t>();
    a.mats = s->mats.buf.as<Material>();
    a.prims0 = s->prims0.buf.as<float4>();
    a.lights = s->lights.buf.as<LightRec>();
    a.rtl = s->rtl;
    a.colors = s->colors.buf.as<ptgpu_vec>();
    a.pixels = s->pixels.buf.as<uint32_t>();
    a.seeds = s->seeds.buf.as<uint32_t>();
    a.pixel_counter = s->d_pixctr.as<unsigned int>();
    a.scenes = s->d_recs.as<BatchScene>();
    a.pix_start = s->d_pix_start.as<int64_t>();
    a.n_scenes = S;
    SK(launch_render_batch(a, 128, stack, grid, s->stream));
    int32_t err = 0;
    SK(cudaMemcpyAsync(&err, s->d_err.p, sizeof(err), cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->steps++;
    }
    std::vector<std::shared_ptr<Request>> keep;
    for (int k = 0, j = 0; k < A; ++k) {
        std::shared_ptr<Request> q = s->active[k];
        if (j < S && sel[j] == k) {
            q->done_passes += recs[j].passes;
            q->steps++;
            ++j;
        } else {
            keep.push_back(q);              // not in this step: waits for a later one
            continue;
        }
        if (q->done_passes < q->r.spp && !err) { keep.push_back(q); continue; }
        const int64_t px = (int64_t)q->r.width * q->r.height;
        q->pixels.resize(px);
        q->colors.resize(px);
        cudaError_t e = cudaMemcpyAsync(q->pixels.data(), s->pixels.buf.as<uint32_t>() + q->pix_base,
                                        px * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(q->colors.data(), s->colors.buf.as<ptgpu_vec>() + q->pix_base,
                                px * sizeof(ptgpu_vec), cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        s->pix_slots.release(q->pix_base, px);
        scene_of(s, q->r.scene).users--;
        int st = PTGPU_OK;
        if (e != cudaSuccess) st = cuda_fail(e, "result copy");
        else if (err & 1) st = record_error(PTGPU_E_RANGE, "traversal stack overflow");
        finish(s, q, st);
    }
    if (err) cudaMemsetAsync(s->d_err.p, 0, 16, s->stream);
    s->active.swap(keep);
    s->n_active = (int)s->active.size();
    return PTGPU_OK;
}

void worker_main(ptgpu_server *s) {
    cudaSetDevice(s->device);
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] {
                return s->stop || !s->pending.empty() || !s->active.empty() || !s->previews.empty();
            });
            if (s->stop && s->pending.empty() && s->active.empty()) {
                lk.unlock();
                serve_previews(s);
                return;
            }
        }
        serve_previews(s);
        admit(s);
        if (s->active.empty()) {
            // nothing admissible now: wait for a new submission
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
            continue;
        }
        const int st = step(s);
        if (st != PTGPU_OK) {
            for (auto &q : s->active) {
                s->pix_slots.release(q->pix_base, (int64_t)q->r.width * q->r.height);
                scene_of(s, q->r.scene).users--;
                finish(s, q, st);
            }
            s->active.clear();
            s->n_active = 0;
        }
    }
}

}  // namespace

extern "C" {

int ptgpu_server_create(int32_t device, int64_t budget_bytes, int32_t quantum, uint32_t flags,
                        ptgpu_server **out) {
    if (!out) return record_error(PTGPU_E_INVAL, "null output");
    if (budget_bytes <= 0) return record_error(PTGPU_E_INVAL, "budget must be positive");
    if (quantum < 0) return record_error(PTGPU_E_INVAL, "quantum must be >= 0");
    *out = nullptr;
    ptgpu_server *s = new ptgpu_server();
    s->device = device;
    s->budget = budget_bytes;
    s->quantum = quantum ? quantum : 4;
    s->rtl = (flags & PTGPU_FLAG_ARGS_RTL) ? 1 : 0;
    s->fill_cap = (flags & PTGPU_SERVER_ALL_ACTIVE) == 0;
    s->nodes.elem = 4 * sizeof(float4);
    s->prims.elem = 3 * sizeof(float4);
    s->prim_id.elem = sizeof(int32_t);
    s->mats.elem = sizeof(Material);
    s->prims0.elem = 3 * sizeof(float4);
    s->lights.elem = sizeof(LightRec);
    s->colors.elem = sizeof(ptgpu_vec);
    s->pixels.elem = sizeof(uint32_t);
    s->seeds.elem = 2 * sizeof(uint32_t);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = s->d_pixctr.ensure(16);
    if (e == cudaSuccess) e = s->d_err.ensure(16);
    if (e == cudaSuccess) e = s->d_depth.ensure(16);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_err.p, 0, 16, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        const int st = cuda_fail(e, "server set-up");
        if (s->stream) cudaStreamDestroy(s->stream);
        delete s;
        return st;
    }
    s->worker = std::thread(worker_main, s);
    *out = s;
    return PTGPU_OK;
}

int ptgpu_server_destroy(ptgpu_server *s) {
    if (!s) return PTGPU_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    Arena *as[] = {&s->nodes, &s->prims, &s->prim_id, &s->mats, &s->prims0, &s->lights,
                   &s->colors, &s->pixels, &s->seeds};
    for (Arena *a : as) a->buf.release();
    DevBuf *bufs[] = {&s->d_recs, &s->d_pix_start, &s->d_pixctr, &s->d_err, &s->d_seg, &s->d_depth,
                      &s->s_shapes, &s->s_verts,
                      &s->s_type, &s->s_aabbs, &s->s_keys, &s->s_keys_alt, &s->s_keys_tmp,
                      &s->s_vals_alt, &s->s_vals_tmp, &s->s_sorted, &s->s_status, &s->s_state,
                      &s->s_bb, &s->s_arr, &s->s_btn, &s->s_btl, &s->s_tcount, &s->s_tcost};
    for (DevBuf *d : bufs) d->release();
    s->ingest.release();
    cudaStreamDestroy(s->stream);
    delete s;
    return PTGPU_OK;
}

static int ptgpu_server_add_scene_body(ptgpu_server *s, const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt,
                           uint32_t build_flags, int32_t *scene) {
    if (!s || !shapes) return record_error(PTGPU_E_INVAL, "null argument");
    if (n < 2) return record_error(PTGPU_E_INVAL, "a served scene needs at least 2 shapes");
    if (n >= (1u << 29)) return record_error(PTGPU_E_RANGE, "scene too large");
    if (build_flags & PTGPU_FLAG_MORTON_DELTA) return record_error(PTGPU_E_INVAL, "build flag not supported");
    for (uint32_t i = 0; i < n; ++i)
        if (shapes[i].type != PTGPU_SPHERE && shapes[i].type != PTGPU_TRIANGLE)
            return record_error(PTGPU_E_INVAL, "shape " + std::to_string(i) + " has an unknown type");
    auto e = std::make_unique<SceneEntry>();
    e->shapes.assign(shapes, shapes + n);
    e->n_shapes = n;
    e->light_cnt = light_cnt;
    e->build_flags = build_flags;
    make_lights(shapes, n, light_cnt, e->lights);
    e->n_lights = (int)e->lights.size();
    std::lock_guard<std::mutex> lk(s->mu);
    s->scenes.push_back(std::move(e));
    if (scene) *scene = (int32_t)s->scenes.size() - 1;
    return PTGPU_OK;
}

static int ptgpu_server_add_scene_file_body(ptgpu_server *s, const char *path, uint32_t build_flags, int32_t *scene) {
    if (!s || !path) return record_error(PTGPU_E_INVAL, "null argument");
    if (build_flags & PTGPU_FLAG_MORTON_DELTA) return record_error(PTGPU_E_INVAL, "build flag not supported");
    // read once to check the file and count its shapes and lights; the
    // scene is read again whenever it has to be built
    CompactScene cs;
    std::string err;
    int st = read_scene_compact(path, 1, 1, cs, err);
    if (st != PTGPU_OK) return record_error(st, err);
    if (cs.walllight) add_wall_light(cs);
    const int64_t n = cs.count();
    if (n < 2) return record_error(PTGPU_E_INVAL, "a served scene needs at least 2 shapes");
    if (n >= (1 << 29)) return record_error(PTGPU_E_RANGE, "scene too large");
    auto e = std::make_unique<SceneEntry>();
    e->path = path;
    e->n_shapes = n;
    e->light_cnt = cs.light_cnt;
    e->n_lights = (int)compact_light_count(cs);
    e->build_flags = build_flags;
    std::lock_guard<std::mutex> lk(s->mu);
    s->scenes.push_back(std::move(e));
    if (scene) *scene = (int32_t)s->scenes.size() - 1;
    return PTGPU_OK;
}

static int ptgpu_server_submit_body(ptgpu_server *s, const ptgpu_request *r, int64_t *ticket) {
    if (!s || !r || !ticket) return record_error(PTGPU_E_INVAL, "null argument");
    if (r->width <= 0 || r->height <= 0 || (int64_t)r->width * r->height > (1ll << 28))
        return record_error(PTGPU_E_INVAL, "bad image size");
    if (r->spp <= 0) return record_error(PTGPU_E_INVAL, "spp must be positive");
    if (r->max_depth < 0 || r->max_depth > 1024) return record_error(PTGPU_E_INVAL, "bad max_depth");
    auto q = std::make_shared<Request>();
    q->r = *r;
    q->r.camera.width = (float)r->width;
    q->r.camera.height = (float)r->height;
    update_camera(&q->r.camera);
    q->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (r->scene < 0 || r->scene >= (int)s->scenes.size())
            return record_error(PTGPU_E_INVAL, "no such scene");
        q->ticket = s->next_ticket++;
        s->tickets[q->ticket] = q;
        s->pending.push_back(q);
        *ticket = q->ticket;
    }
    s->cv_work.notify_all();
    return PTGPU_OK;
}

int ptgpu_server_wait(ptgpu_server *s, int64_t ticket, uint32_t *pixels, ptgpu_vec *colors,
                      ptgpu_request_stats *stats) {
    if (!s) return record_error(PTGPU_E_INVAL, "null server");
    std::shared_ptr<Request> q;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->tickets.find(ticket);
        if (it == s->tickets.end()) return record_error(PTGPU_E_INVAL, "unknown ticket");
        q = it->second;
        s->cv_done.wait(lk, [&] { return q->finished; });
        s->tickets.erase(ticket);
    }
    if (stats) {
        stats->queued_ms = q->status == PTGPU_OK ? ms_since(q->t_submit, q->t_admit) : 0.0;
        stats->latency_ms = ms_since(q->t_submit, q->t_done);
        stats->steps = q->steps;
        stats->built = q->built;
    }
    if (q->status == PTGPU_E_CANCELED) return record_error(q->status, "request cancelled");
    if (q->status != PTGPU_OK) return record_error(q->status, "request failed");
    if (pixels) std::memcpy(pixels, q->pixels.data(), q->pixels.size() * sizeof(uint32_t));
    if (colors) std::memcpy(colors, q->colors.data(), q->colors.size() * sizeof(ptgpu_vec));
    return PTGPU_OK;
}

int ptgpu_server_cancel(ptgpu_server *s, int64_t ticket) {
    if (!s) return record_error(PTGPU_E_INVAL, "null server");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->tickets.find(ticket);
        if (it == s->tickets.end()) return record_error(PTGPU_E_INVAL, "unknown ticket");
        it->second->cancel = true;
    }
    s->cv_work.notify_all();
    return PTGPU_OK;
}

int ptgpu_server_preview(ptgpu_server *s, int64_t ticket, uint32_t *pixels, ptgpu_vec *colors,
                         int32_t *passes_done) {
    if (!s) return record_error(PTGPU_E_INVAL, "null server");
    auto job = std::make_shared<PreviewJob>();
    job->pixels = pixels;
    job->colors = colors;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->tickets.find(ticket);
        if (it == s->tickets.end()) return record_error(PTGPU_E_INVAL, "unknown ticket");
        job->q = it->second;
        s->previews.push_back(job);
        s->cv_work.notify_all();
        s->cv_done.wait(lk, [&] { return job->done; });
    }
    if (passes_done) *passes_done = job->passes;
    if (job->status == PTGPU_E_STATE) return record_error(PTGPU_E_STATE, "request not admitted yet");
    if (job->status != PTGPU_OK) return record_error(job->status, "request failed or preview copy failed");
    return PTGPU_OK;
}

int ptgpu_server_info_get(ptgpu_server *s, ptgpu_server_info *info) {
    if (!s || !info) return record_error(PTGPU_E_INVAL, "null argument");
    std::memset(info, 0, sizeof(*info));
    std::lock_guard<std::mutex> lk(s->mu);
    info->budget_bytes = s->budget;
    info->bytes_in_use = s->bytes_in_use();
    info->requests_done = s->done_count;
    info->builds = s->builds;
    info->evictions = s->evictions;
    info->steps = s->steps;
    int resident = 0;
    for (const auto &e : s->scenes) resident += e->resident ? 1 : 0;
    info->resident_scenes = resident;
    info->active_requests = s->n_active.load();
    info->pending_requests = (int32_t)s->pending.size();
    info->quantum = s->quantum;
    info->samples_done = s->samples_done;
    info->shape_slots_used = s->shape_slots_used;
    info->pixel_slots_used = s->pixel_slots_used;
    info->light_slots_used = s->light_slots_used;
    return PTGPU_OK;
}

}  // extern "C"

// C entry points: no C++ exception crosses the C ABI
int ptgpu_server_add_scene(ptgpu_server *s, const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt,
                           uint32_t build_flags, int32_t *scene) {
    try {
        return ptgpu_server_add_scene_body(s, shapes, n, light_cnt, build_flags, scene);
    } catch (const std::bad_alloc &) {
        return record_error(PTGPU_E_OOM, "out of host memory");
    } catch (const std::exception &e) {
        return record_error(PTGPU_E_INVAL, std::string("unexpected error: ") + e.what());
    }
}

int ptgpu_server_add_scene_file(ptgpu_server *s, const char *path, uint32_t build_flags, int32_t *scene) {
    try {
        return ptgpu_server_add_scene_file_body(s, path, build_flags, scene);
    } catch (const std::bad_alloc &) {
        return record_error(PTGPU_E_OOM, "out of host memory");
    } catch (const std::exception &e) {
        return record_error(PTGPU_E_INVAL, std::string("unexpected error: ") + e.what());
    }
}

int ptgpu_server_submit(ptgpu_server *s, const ptgpu_request *r, int64_t *ticket) {
    try {
        return ptgpu_server_submit_body(s, r, ticket);
    } catch (const std::bad_alloc &) {
        return record_error(PTGPU_E_OOM, "out of host memory");
    } catch (const std::exception &e) {
        return record_error(PTGPU_E_INVAL, std::string("unexpected error: ") + e.what());
    }
}
