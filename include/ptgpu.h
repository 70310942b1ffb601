/*
 * ptgpu.h -- C ABI of the GB300 (sm_103a) LBVH builder and path tracer.
 *
 * This header is the drop-in boundary for PTGPU_PC's hot path: the LBVH build
 * (CLBVH + BVH.cl), the host KD-tree build (KDTree.cpp), the scene loader
 * (displayfunc.cpp Read/ReadTxt/ReadScene, UpdateCamera) and the per-pixel
 * radiance path tracer (rendering_kernel.cl RadianceGPU).  Every struct below
 * keeps the byte layout of the reference struct it mirrors (checked by the
 * static asserts at the end), so arrays produced by the reference can be passed
 * in unchanged and arrays returned here can be handed to reference code.
 *
 * Conventions
 *  - Every function returns an int status: PTGPU_OK (0) or a negative
 *    PTGPU_E_* code.  ptgpu_status_string() names it; ptgpu_last_error()
 *    gives a one-line message for the last failure on the calling thread.
 *  - Host pointers only; no CUDA or torch types in any signature.  Device
 *    memory is owned by the context.  A stream may be supplied as an opaque
 *    handle (cudaStream_t cast to void*) through ptgpu_config.stream.
 *  - One context per thread.  Device-side waits are bounded and surface as
 *    PTGPU_E_TIMEOUT; the context stays usable afterwards.
 */
#ifndef PTGPU_H
#define PTGPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PTGPU_ABI_VERSION 1

/* ---- status codes -------------------------------------------------------- */
#define PTGPU_OK           0
#define PTGPU_E_INVAL     -1  /* bad argument, bad count, unsupported mode      */
#define PTGPU_E_OOM       -2  /* device or host allocation failed               */
#define PTGPU_E_DEVICE    -3  /* CUDA error (sticky errors need a new context)  */
#define PTGPU_E_TIMEOUT   -4  /* a bounded device wait gave up                  */
#define PTGPU_E_IO        -5  /* scene file missing or malformed                */
#define PTGPU_E_RANGE     -6  /* result does not fit the reference layout       */
#define PTGPU_E_STATE     -7  /* call out of order (e.g. draw before build)     */
#define PTGPU_E_CANCELED  -8  /* a served request was cancelled                 */

/* ---- reference constants (include/geom.h:29-35, clheader.h:9-15) --------- */
#define PTGPU_EPSILON      0.01f
#define PTGPU_MAX_DEPTH    6
#define PTGPU_ACCEL_NONE   0   /* ACCELSTR 0: brute force                   */
#define PTGPU_ACCEL_BVH    1   /* ACCELSTR 1: LBVH (the reference default)  */
#define PTGPU_ACCEL_KDTREE 2   /* ACCELSTR 2: KD tree (KDTree::build)       */

/* ---- shared geometry types (include/geom.h:48-91, vec.h:27-29) ----------- */
typedef struct { float x, y, z; } ptgpu_vec;                 /* Vec      */
typedef struct { ptgpu_vec o, d; } ptgpu_ray;                /* Ray      */
typedef struct { float rad; ptgpu_vec p; } ptgpu_sphere;     /* Sphere   */
typedef struct { ptgpu_vec p1, p2, p3; } ptgpu_triangle;     /* Triangle */
typedef struct {                                             /* Bound    */
    float min_x, max_x, min_y, max_y, min_z, max_z;
} ptgpu_bound;

enum { PTGPU_SPHERE = 0, PTGPU_TRIANGLE = 1 };            /* tagType     */
enum { PTGPU_DIFF = 0, PTGPU_SPEC = 1, PTGPU_REFR = 2 };  /* enum Refl   */

typedef struct {                                             /* Shape    */
    int32_t type;                 /* PTGPU_SPHERE / PTGPU_TRIANGLE  @0  */
    union { ptgpu_triangle t; ptgpu_sphere s; } g;       /*          @4  */
    ptgpu_vec e, c;               /* emission @40, colour @52             */
    int32_t refl;                 /* PTGPU_DIFF/SPEC/REFR           @64 */
    int32_t index;                /*                                @68 */
    uint32_t morton_code;         /*                                @72 */
    ptgpu_bound b;                /*                                @76 */
    float area;                   /*                                @100*/
} ptgpu_shape;

/* include/camera.h:29-38 */
typedef struct {
    ptgpu_vec orig, target;       /* target is read but unused (UpdateCamera) */
    float pitch, yaw;
    float width, height;
    ptgpu_vec dir, x, y;          /* filled by ptgpu_update_camera */
} ptgpu_camera;

/* include/BVHNodeGPU.h:4-16.  btn[N-1] internal nodes, btl[N] leaves. */
typedef struct {
    int32_t min, max;             /* leaf range of an internal node         */
    int32_t nShape;               /* shape id (leaves)                      */
    int32_t leaf;                 /* 0 internal, 2 "has a leaf child", -1 leaf */
    int32_t nLeft, nRight, nParent;
    ptgpu_bound bound;
    float cost, area;
} ptgpu_bvh_node;

/* include/KDNodeGPU.h:4-14.  Heap layout, root at index 1. */
typedef struct {
    int16_t leaf;
    int16_t nLeft, nRight, nParent;
    ptgpu_bound bound;
    int16_t min, max;             /* [min,max) into the kn index list       */
} ptgpu_kd_node;

/* The same KD tree with 32-bit fields, for trees the int16 heap above cannot
 * express (KDNodeGPU overflows past 32,767 heap slots; an 82k-shape scene needs
 * 2^18).  Nodes breadth-first, root at index 0, children at nLeft/nRight and
 * the parent at nParent (-1 where there is none); a leaf owns [min, max) of the
 * kn index list, which is the heap export's kn. */
typedef struct {
    int32_t leaf;                 /* 1 leaf, 0 internal                     */
    int32_t nLeft, nRight, nParent;
    ptgpu_bound bound;
    int32_t min, max;
} ptgpu_kd_node_wide;

/* ---- context -------------------------------------------------------------- */
typedef struct ptgpu_ctx ptgpu_ctx;

typedef struct {
    int32_t device;        /* CUDA device ordinal                               */
    int32_t accel;         /* PTGPU_ACCEL_*: runtime form of ACCELSTR           */
    int32_t max_depth;     /* MAX_DEPTH; 0 selects the reference value 6        */
    int32_t width, height; /* image size; sets camera.width/height              */
    int32_t block_size;    /* render block size; 0 = default                    */
    int32_t flags;         /* PTGPU_FLAG_*                                       */
    int32_t rr_depth;      /* 0: paths end only at max_depth (the reference);
                              d > 0: throughput Russian roulette from the hit
                              at depth d (0-based) on: a path continues with
                              probability p = min(max(throughput), 1) and its
                              throughput is divided by p (one random per
                              roll, drawn after the bounce's).  Lane tracer
                              only: with PTGPU_FLAG_WAVEFRONT, E_INVAL.       */
    void   *stream;        /* optional cudaStream_t; NULL = context-owned stream */
} ptgpu_config;

/* build / render flags */
#define PTGPU_FLAG_WAVEFRONT     0x1  /* render with the queue-based wavefront  */
#define PTGPU_FLAG_MORTON_DELTA  0x2  /* reserved (a Karras split on the Morton
                                         keys); ptgpu_build answers E_INVAL     */
#define PTGPU_FLAG_TREELET       0x4  /* treelet reoptimisation after refit     */
#define PTGPU_FLAG_WIDE_TRAVERSAL 0x10 /* traverse 4-wide nodes collapsed from
                                         the 2-wide ones (default: 2-wide)      */
#define PTGPU_FLAG_ARGS_RTL      0x8  /* draw the two randoms of a light sample
                                         right-to-left (the order g++ gives the
                                         reference source; the default is the
                                         left-to-right order of OpenCL/clang)   */
#define PTGPU_FLAG_KD_HOST       0x20 /* build the KD tree with the sequential host
                                         code instead of the GPU (same tree)     */
#define PTGPU_FLAG_ROW_ORDER     0x40 /* hand pixels out in row order on every
                                         frame (default: from the second frame on,
                                         in decreasing work of the frame before;
                                         results are the same either way)      */
/* build flag field: rounds of the treelet stage (bits 8-11; 0 = one round,
 * the single launch of CLBVH::optimize, CLBVH.cpp:318-350).  Each round runs
 * over the tree the previous one left; Karras & Aila use three. */
#define PTGPU_TREELET_SWEEPS(n)  ((uint32_t)((n) & 0xF) << 8)

int  ptgpu_create(const ptgpu_config *cfg, ptgpu_ctx **out);
int  ptgpu_destroy(ptgpu_ctx *ctx);
const char *ptgpu_status_string(int status);
const char *ptgpu_last_error(void);
int  ptgpu_abi_version(void);

/* ---- scene ---------------------------------------------------------------- */
/* Read(fileName, &walllight) + AddWallLight (displayfunc.cpp:717-730,
 * smallptGPU.cpp:1448-1459): ".txt", ".scn" dispatch by extension.  Sets the
 * context's shapes, light count and camera (orig/target, pitch=yaw=0).        */
int  ptgpu_read_scene(ptgpu_ctx *ctx, const char *path, int32_t *walllight);
/* The same scene as ptgpu_read_scene (same shapes byte for byte, light count,
 * camera, walllight) without a host copy of the shape array: OBJ models are
 * read on several host threads into vertex and index arrays, copied as they
 * are, and expanded into Shape records on the device (ReadTxt's model
 * branch, displayfunc.cpp:395-420, done on the GPU).  Calls that need the
 * shapes on the host later (ptgpu_get_shapes before a BVH build, the host KD
 * build) copy them back once. */
int  ptgpu_stream_scene(ptgpu_ctx *ctx, const char *path, int32_t *walllight);
/* Copies n shapes in (the global `shapes`/`shapeCnt`/`lightCnt`). */
int  ptgpu_set_shapes(ptgpu_ctx *ctx, const ptgpu_shape *shapes, uint32_t n,
                      uint32_t light_cnt);
int  ptgpu_get_shape_count(ptgpu_ctx *ctx, uint32_t *n, uint32_t *light_cnt);
/* Copies the shapes out; after a BVH build index/morton_code/b are filled
 * as CLBVH::CLBVH leaves them (CLBVH.cpp:98-164). */
int  ptgpu_get_shapes(ptgpu_ctx *ctx, ptgpu_shape *out, uint32_t n);

/* UpdateCamera (displayfunc.cpp:732-756): pure host function. */
int  ptgpu_update_camera(ptgpu_camera *cam);
/* Sets the render camera; width/height are forced to the context's size and
 * the basis is recomputed with ptgpu_update_camera (ReInit semantics). */
int  ptgpu_set_camera(ptgpu_ctx *ctx, const ptgpu_camera *cam);
int  ptgpu_get_camera(ptgpu_ctx *ctx, ptgpu_camera *cam);

/* ---- acceleration structures ---------------------------------------------- */
/* BuildBVH (smallptGPU.cpp:1462-1472) or BuildKDtree (:1477-1493). */
int  ptgpu_build(ptgpu_ctx *ctx, int32_t accel, uint32_t flags);
/* CLBVH::getTrees (CLBVH.cpp:357-366): copies btn[N-1] and btl[N] out. */
int  ptgpu_get_bvh(ptgpu_ctx *ctx, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl);
/* KDTree::getTrees (KDTree.cpp:257-270).  Size query: pass NULL buffers to
 * get *kng_cnt / *kn_cnt.  PTGPU_E_RANGE if the heap overflows int16. */
int  ptgpu_get_kdtree(ptgpu_ctx *ctx, ptgpu_kd_node *kng, int32_t *kng_cnt,
                      int32_t *kn, int32_t *kn_cnt);
/* KDTree::getTrees (KDTree.cpp:257-270) without the int16 limit: the tree as
 * ptgpu_kd_node_wide records (breadth-first, the heap's node order with its
 * empty slots left out) and the same kn list.  Size query: pass NULL buffers
 * to get *node_cnt / *kn_cnt; E_INVAL when a buffer is smaller than that. */
int  ptgpu_get_kdtree_wide(ptgpu_ctx *ctx, ptgpu_kd_node_wide *nodes, int32_t *node_cnt,
                           int32_t *kn, int32_t *kn_cnt);
/* Installs caller-built BVH arrays (the ReInit upload, smallptGPU.cpp:1145-1148). */
int  ptgpu_set_bvh(ptgpu_ctx *ctx, const ptgpu_bvh_node *btn,
                   const ptgpu_bvh_node *btl, uint32_t n);
/* No counterpart in the reference (its look-back-free host sort never
 * waits).  The radix sort's decoupled look-back waits for earlier tiles; a
 * tile that has polled `polls` times (about 32 ns apart) without an answer
 * gives up and ptgpu_build returns PTGPU_E_TIMEOUT, leaving the context
 * usable.  The default is PTGPU_WAIT_LIMIT_DEFAULT; 0 gives up at the first
 * wait, so any build of more than one sort tile (5,120 shapes) times out --
 * a way to exercise the error path without a fault. */
#define PTGPU_WAIT_LIMIT_DEFAULT 4194304u
int  ptgpu_set_wait_limit(ptgpu_ctx *ctx, uint32_t polls);
/* Last build's device time in milliseconds (CUDA events on the ctx stream). */
int  ptgpu_last_build_ms(ptgpu_ctx *ctx, float *ms);

/* ---- rendering ------------------------------------------------------------ */
/* Seeds: 2*W*H words, seed0/seed1 interleaved per pixel (AllocateBuffers,
 * smallptGPU.cpp:185-217).  ptgpu_make_seeds fills them from a 64-bit master
 * seed (SplitMix64, low 32 bits, clamped to >= 2 like the reference). */
int  ptgpu_make_seeds(uint64_t master_seed, uint32_t *seeds, uint32_t count);
int  ptgpu_set_seeds(ptgpu_ctx *ctx, const uint32_t *seeds);
int  ptgpu_get_seeds(ptgpu_ctx *ctx, uint32_t *seeds);
/* Resets the progressive sample counter (ReInit: currentSample = 0). */
int  ptgpu_reset_accumulation(ptgpu_ctx *ctx);
/* DrawFrame (smallptGPU.cpp:918-1126): runs `passes` RadianceGPU passes and
 * returns the RGBA8 pixel buffer (library-owned, valid until the next call). */
int  ptgpu_draw_frame(ptgpu_ctx *ctx, uint32_t passes, const uint32_t **pixels_out);
/* Enqueues `passes` passes without any host copy (device-resident timing). */
int  ptgpu_render_async(ptgpu_ctx *ctx, uint32_t passes);
/* Runs `passes` passes like ptgpu_render_async with traversal counters on and
 * synchronises: stats[0..5] = extension node visits, extension primitive
 * tests, shadow node visits, shadow primitive tests, extension queries,
 * shadow queries.  For the benchmark's bytes-moved model. */
int  ptgpu_render_stats(ptgpu_ctx *ctx, uint32_t passes, uint64_t *stats);
int  ptgpu_synchronize(ptgpu_ctx *ctx);
/* The float accumulation buffer `colors` (W*H Vec, row-flipped as in
 * RadianceGPU) and the packed pixels. */
int  ptgpu_get_colors(ptgpu_ctx *ctx, ptgpu_vec *colors);
int  ptgpu_get_pixels(ptgpu_ctx *ctx, uint32_t *pixels);
int  ptgpu_get_current_sample(ptgpu_ctx *ctx, int32_t *current_sample);

/* ---- closest-hit queries ---------------------------------------------------- */
/* Intersect (rendering_kernel.cl:194-363) for n rays with the current accel:
 * t[i] (1e20 on a miss), id[i] (shape id), hit[i] (0/1). */
int  ptgpu_trace_closest(ptgpu_ctx *ctx, const ptgpu_ray *rays, uint32_t n,
                         float *t, uint32_t *id, int32_t *hit);

/* Device-resident variants for benchmarking: the arrays live in memory the
 * caller allocated with CUDA on the context's device. */
int  ptgpu_trace_closest_device(ptgpu_ctx *ctx, const ptgpu_ray *d_rays,
                                uint32_t n, float *d_t, uint32_t *d_id,
                                int32_t *d_hit);
/* ptgpu_trace_closest_device with traversal counters on, synchronised:
 * stats[0] = node visits, stats[1] = primitive tests over all n rays (the
 * benchmark's bytes-per-ray model; no counterpart in the reference). */
int  ptgpu_trace_closest_stats(ptgpu_ctx *ctx, const ptgpu_ray *d_rays,
                               uint32_t n, float *d_t, uint32_t *d_id,
                               int32_t *d_hit, uint64_t *stats);
int  ptgpu_get_stream(ptgpu_ctx *ctx, void **stream);

/* ---- batched scenes ------------------------------------------------------- */
/* No counterpart in the reference (its process renders one scene).  A batch
 * holds many scenes -- shapes, camera, image size, passes, seeds each -- and
 * builds every scene's LBVH in one segmented pass of the build kernels (one
 * radix sort over all scenes' keys), then renders all scenes' pixels in one
 * persistent launch replayed from a CUDA graph.  A scene's BVH arrays,
 * colours and pixels are the ones a single-scene context produces from the
 * same inputs and build flags.  BVH only; binary traversal; up to 256 scenes
 * of at least 2 shapes each.  One thread per batch.                          */
typedef struct ptgpu_batch ptgpu_batch;

typedef struct {
    const ptgpu_shape *shapes;  /* n shapes, copied by ptgpu_batch_add           */
    uint32_t n, light_cnt;      /* as ptgpu_set_shapes                          */
    ptgpu_camera camera;        /* orig/pitch/yaw; UpdateCamera runs on add     */
    int32_t width, height;
    int32_t passes;             /* passes of one ptgpu_batch_render              */
    int32_t max_depth;          /* 0 selects PTGPU_MAX_DEPTH                     */
    const uint32_t *seeds;      /* 2*width*height seeds, copied                  */
} ptgpu_scene;

typedef struct {
    float build_ms;             /* last ptgpu_batch_build: device time            */
    float render_ms;            /* last ptgpu_batch_render: device time           */
    double samples;             /* samples of one render (sum of W*H*passes)      */
    int32_t block, refill, stack; /* launch settings in use (ptgpu_batch_tune)    */
    int32_t tree_depth;         /* deepest leaf over all scenes' trees           */
    int64_t shapes;             /* shapes over all scenes                         */
} ptgpu_batch_info;

int  ptgpu_batch_create(int32_t device, uint32_t flags, ptgpu_batch **out); /* flags: PTGPU_FLAG_ARGS_RTL */
int  ptgpu_batch_destroy(ptgpu_batch *b);
int  ptgpu_batch_add(ptgpu_batch *b, const ptgpu_scene *scene, int32_t *scene_id);
/* Uploads every scene and builds all trees (build flags as ptgpu_build with
 * PTGPU_ACCEL_BVH: PTGPU_FLAG_TREELET, PTGPU_TREELET_SWEEPS).  Resets the
 * accumulation. */
int  ptgpu_batch_build(ptgpu_batch *b, uint32_t flags);
/* Times short one-pass renders of the batch over block sizes (64, 96, 128)
 * and refill thresholds (16, 20, 24 of 32 lanes), keeps the fastest, and
 * restores the seeds; the stack depth (32, 64 or 128) follows the deepest tree.
 * Resets the accumulation. */
int  ptgpu_batch_tune(ptgpu_batch *b);
/* One frame: each scene's `passes` passes, accumulated onto its running mean
 * (the first frame after build/reset overwrites).  Returns when done. */
int  ptgpu_batch_render(ptgpu_batch *b);
int  ptgpu_batch_reset(ptgpu_batch *b);
int  ptgpu_batch_get_pixels(ptgpu_batch *b, int32_t scene, uint32_t *pixels);   /* W*H RGBA8 */
int  ptgpu_batch_get_colors(ptgpu_batch *b, int32_t scene, ptgpu_vec *colors);  /* W*H, row-flipped */
int  ptgpu_batch_get_bvh(ptgpu_batch *b, int32_t scene, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl);
int  ptgpu_batch_info_get(ptgpu_batch *b, ptgpu_batch_info *info);

/* ---- serving --------------------------------------------------------------- */
/* No counterpart in the reference.  A server owns a worker thread that runs
 * render requests with continuous batching: requests wait in arrival order,
 * are admitted while their scene and their accumulation buffers fit the HBM
 * budget, and every step renders up to `quantum` more passes of every
 * admitted request in one launch, so requests that arrive while others run
 * join at the next step.  Built scenes stay resident between requests under
 * LRU (keyed by scene id) and are rebuilt after eviction.  A request's pixels
 * depend only on its scene, camera, size, passes and seed: they equal a
 * single-scene context's draw_frame(spp) after set_seeds(ptgpu_make_seeds(
 * seed, 2*W*H)), alone or in any mix.  Submit and wait are thread-safe.     */
typedef struct ptgpu_server ptgpu_server;

typedef struct {
    int32_t scene;              /* id from ptgpu_server_add_scene                */
    int32_t width, height;
    int32_t spp;                /* passes to render                              */
    int32_t max_depth;          /* 0 selects PTGPU_MAX_DEPTH                     */
    int32_t pad;
    uint64_t seed;              /* master seed of the request's seed streams     */
    ptgpu_camera camera;        /* orig/pitch/yaw; UpdateCamera runs on submit   */
} ptgpu_request;

typedef struct {
    double queued_ms;           /* submit -> admission                           */
    double latency_ms;          /* submit -> result ready                        */
    int32_t steps;              /* render steps the request took part in         */
    int32_t built;              /* 1: its scene was built for it (cache miss)    */
} ptgpu_request_stats;

typedef struct {
    int64_t budget_bytes, bytes_in_use;
    int64_t requests_done, builds, evictions, steps;
    int32_t resident_scenes, active_requests, pending_requests, quantum;
    double samples_done;
    /* slots held now: shape slots of resident scenes, pixel slots of admitted
     * requests, light records of resident scenes */
    int64_t shape_slots_used, pixel_slots_used, light_slots_used;
} ptgpu_server_info;

/* Steps.  By default each step renders the admitted requests oldest first
 * while their pixels add up to at most one filling of the GPU (four pixels
 * per resident render lane); the oldest is always rendered, the others wait
 * for a later step.  A request that fills the GPU by itself then runs alone,
 * as in a first-come queue, while small ones still share steps.  With this
 * server flag every admitted request takes part in every step instead: a
 * few percent more samples per second, but requests that arrive during a
 * large one slow it down (a longer p99). */
#define PTGPU_SERVER_ALL_ACTIVE  0x100

int  ptgpu_server_create(int32_t device, int64_t budget_bytes, int32_t quantum, uint32_t flags,
                         ptgpu_server **out);  /* flags: PTGPU_FLAG_ARGS_RTL, PTGPU_SERVER_ALL_ACTIVE;
                                                  quantum 0 = 4 */
int  ptgpu_server_destroy(ptgpu_server *s);    /* finishes admitted work first */
/* Registers a scene (copied); built on its first request with build_flags. */
int  ptgpu_server_add_scene(ptgpu_server *s, const ptgpu_shape *shapes, uint32_t n,
                            uint32_t light_cnt, uint32_t build_flags, int32_t *scene);
/* A scene by its file (ptgpu_read_scene's formats, wall light included when
 * the file asks for it): read once here to check it and count its shapes,
 * then read again -- models expanded on the device, as ptgpu_stream_scene
 * does -- every time it has to be built (first use, or after eviction); no
 * host copy of its shapes is kept.  The file's camera is not used (requests
 * carry theirs).  Requests on it render as on ptgpu_server_add_scene with
 * ptgpu_read_scene's shapes. */
int  ptgpu_server_add_scene_file(ptgpu_server *s, const char *path, uint32_t build_flags,
                                 int32_t *scene);
int  ptgpu_server_submit(ptgpu_server *s, const ptgpu_request *r, int64_t *ticket);
/* Blocks until the request is done, copies its W*H pixels and colours (either
 * may be NULL) and its stats, and forgets the ticket.  PTGPU_E_RANGE: the
 * request can never fit the budget. */
int  ptgpu_server_wait(ptgpu_server *s, int64_t ticket, uint32_t *pixels, ptgpu_vec *colors,
                       ptgpu_request_stats *stats);
int  ptgpu_server_info_get(ptgpu_server *s, ptgpu_server_info *info);
/* No counterpart in the reference (it has no requests).  Cancels a request
 * that has not been waited for: a pending one leaves the queue, an active one
 * ends at the next step boundary, releasing its pixel slots and its hold on
 * its scene; ptgpu_server_wait then returns PTGPU_E_CANCELED.  A request that
 * already finished keeps its result.  Callable from any thread. */
int  ptgpu_server_cancel(ptgpu_server *s, int64_t ticket);
/* No counterpart in the reference.  Progressive preview: copies the
 * request's W*H pixels and colours (either may be NULL) as they stand after
 * its last finished render step, and the passes they hold; a finished request
 * gives its final image.  PTGPU_E_STATE: not admitted yet (no pass rendered).
 * Does not end or reserve the ticket.  Callable from any thread. */
int  ptgpu_server_preview(ptgpu_server *s, int64_t ticket, uint32_t *pixels, ptgpu_vec *colors,
                          int32_t *passes_done);

/* ---- image output ------------------------------------------------------------ */
/* The frame as an image file, encoded on the device and copied out once.
 * PTGPU_IMAGE_PPM: the reference's dump of the display buffer
 * (smallptGPU.cpp:1238-1257): "P3\n<w> <h>\n255\n", then "<r> <g> <b> " for
 * every pixel, rows from the top of the image down, no line breaks.
 * PTGPU_IMAGE_PFM (no counterpart in the reference): the float running mean,
 * "PF\n<w> <h>\n-1.0\n" and RGB float32 little-endian, bottom row first.
 * E_STATE before the first drawn frame. */
#define PTGPU_IMAGE_PPM 0
#define PTGPU_IMAGE_PFM 1
/* into a caller buffer: *size is its capacity in bytes; buf NULL (or too
 * small: E_INVAL) answers the size in *size */
int  ptgpu_encode_image(ptgpu_ctx *ctx, int32_t format, void *buf, uint64_t *size);
int  ptgpu_write_image(ptgpu_ctx *ctx, const char *path, int32_t format);

/* ---- BVH build without device allocation ----------------------------------- */
/* No counterpart in the reference.  The LBVH build of ptgpu_build(ctx,
 * PTGPU_ACCEL_BVH, 0) -- same btn[n-1] / btl[n] bytes -- from n shapes in
 * device memory into node arrays in device memory, all three allocated by the
 * caller on the current device; no context.  For callers that may not let a
 * library allocate device memory (an engine with its own pool or fixed budget,
 * a frame loop that must not stall on cudaMalloc/cudaFree, a plug-in host that
 * forbids it): intermediates live in a fixed array inside the library, so
 * n <= 262144 (PTGPU_E_RANGE beyond).  d_btn holds at least one node when
 * n == 1; nothing is written past btn[max(n-1,1)-1] or btl[n-1].  The first
 * call on a device sets up that device's array: make it before any stream
 * capture.  Calls that overlap on the GPU share the array and race: serialise
 * them.  Enqueued on `stream` (cudaStream_t, NULL = legacy default); every
 * call waits on the host for its build to finish before it returns.  */
int  ptgpu_build_bvh_noalloc(const ptgpu_shape *d_shapes, uint32_t n,
                             ptgpu_bvh_node *d_btn, ptgpu_bvh_node *d_btl,
                             void *stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

/* ---- layout checks against the reference structs -------------------------- */
#ifdef __cplusplus
#define PTGPU_SA(c, m) static_assert(c, m)
#else
#define PTGPU_SA(c, m) _Static_assert(c, m)
#endif
PTGPU_SA(sizeof(ptgpu_vec) == 12, "Vec is 12 bytes");
PTGPU_SA(sizeof(ptgpu_ray) == 24, "Ray is 24 bytes");
PTGPU_SA(sizeof(ptgpu_sphere) == 16, "Sphere is 16 bytes");
PTGPU_SA(sizeof(ptgpu_triangle) == 36, "Triangle is 36 bytes");
PTGPU_SA(sizeof(ptgpu_bound) == 24, "Bound is 24 bytes");
PTGPU_SA(sizeof(ptgpu_shape) == 104, "Shape is 104 bytes");
PTGPU_SA(offsetof(ptgpu_shape, e) == 40, "Shape.e at 40");
PTGPU_SA(offsetof(ptgpu_shape, refl) == 64, "Shape.refl at 64");
PTGPU_SA(offsetof(ptgpu_shape, morton_code) == 72, "Shape.morton_code at 72");
PTGPU_SA(offsetof(ptgpu_shape, b) == 76, "Shape.b at 76");
PTGPU_SA(offsetof(ptgpu_shape, area) == 100, "Shape.area at 100");
PTGPU_SA(sizeof(ptgpu_camera) == 76, "Camera is 76 bytes");
PTGPU_SA(sizeof(ptgpu_bvh_node) == 60, "BVHNodeGPU is 60 bytes");
PTGPU_SA(offsetof(ptgpu_bvh_node, bound) == 28, "BVHNodeGPU.bound at 28");
PTGPU_SA(sizeof(ptgpu_kd_node) == 36, "KDNodeGPU is 36 bytes");
PTGPU_SA(offsetof(ptgpu_kd_node, min) == 32, "KDNodeGPU.min at 32");
PTGPU_SA(sizeof(ptgpu_kd_node_wide) == 48, "wide KD node is 48 bytes");
PTGPU_SA(offsetof(ptgpu_kd_node_wide, min) == 40, "wide KD node min at 40");
/* the batch structs (no reference counterpart): fixed for foreign bindings */
PTGPU_SA(sizeof(ptgpu_scene) == 120, "ptgpu_scene is 120 bytes");
PTGPU_SA(offsetof(ptgpu_scene, camera) == 16, "ptgpu_scene.camera at 16");
PTGPU_SA(offsetof(ptgpu_scene, seeds) == 112, "ptgpu_scene.seeds at 112");
PTGPU_SA(sizeof(ptgpu_batch_info) == 40, "ptgpu_batch_info is 40 bytes");
PTGPU_SA(sizeof(ptgpu_request) == 112, "ptgpu_request is 112 bytes");
PTGPU_SA(offsetof(ptgpu_request, camera) == 32, "ptgpu_request.camera at 32");
PTGPU_SA(sizeof(ptgpu_request_stats) == 24, "ptgpu_request_stats is 24 bytes");
PTGPU_SA(sizeof(ptgpu_server_info) == 96, "ptgpu_server_info is 96 bytes");
#undef PTGPU_SA

#endif /* PTGPU_H */
