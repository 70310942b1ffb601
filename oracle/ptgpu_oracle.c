/*
 * ptgpu_oracle.c -- CPU oracle for the PTGPU_PC hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates the reference algorithms in
 * plain C so the tests can check the GPU library against them, and so the
 * benchmark can time a CPU baseline.  Nothing in the GPU library links or
 * calls it.
 *
 * Float semantics: every expression is evaluated in IEEE binary32, left to
 * right, with no contraction (build with -ffp-contract=off).  That is what the
 * reference's OpenCL kernels compute when the compiler does not fuse, and
 * what the GPU library computes (nvcc -fmad=false).  The OpenCL built-ins the
 * kernels use are given their OpenCL meaning: max/min as fmax/fmin, clamp as
 * fmin(fmax(x, lo), hi), sign(0) = 0.  sin/cos/pow/sqrt come from libm.
 */
#include "ptgpu_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_EPSILON 0.01f
#define ORC_PI 3.14159265358979323846f
#define ORC_INF_T 1e20f

/* ------------------------------------------------------------------------- */
/* vector helpers (include/vec.h:31-47)                                       */
/* ------------------------------------------------------------------------- */
static inline ptgpu_vec v3(float x, float y, float z) { ptgpu_vec v = {x, y, z}; return v; }
static inline ptgpu_vec vsub(ptgpu_vec a, ptgpu_vec b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline ptgpu_vec vadd(ptgpu_vec a, ptgpu_vec b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline ptgpu_vec vmul(ptgpu_vec a, ptgpu_vec b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline ptgpu_vec vsmul(float k, ptgpu_vec b) { return v3(k * b.x, k * b.y, k * b.z); }
static inline float vdot(ptgpu_vec a, ptgpu_vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline ptgpu_vec vcross(ptgpu_vec a, ptgpu_vec b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline ptgpu_vec vnorm(ptgpu_vec v) { float l = 1.f / sqrtf(vdot(v, v)); return vsmul(l, v); }
static inline int viszero(ptgpu_vec v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }
/* OpenCL sign(): 1, -1, or the (signed) zero / 0 for NaN */
static inline float cl_sign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : (x == x ? x : 0.f)); }
static inline float cl_clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
/* include/AccelCommon.h:14-32 and BVH.cl:78-86 (ternary min/max) */
static inline float min2f(float a, float b) { return (a < b) ? a : b; }
static inline float max2f(float a, float b) { return (a > b) ? a : b; }
static inline float min3f(float a, float b, float c) { return min2f(min2f(a, b), c); }
static inline float max3f(float a, float b, float c) { return max2f(max2f(a, b), c); }


/* Deterministic sine/cosine used by the GPU library for the light-sphere and
 * diffuse-bounce angles (arguments in [0, 2*pi)).  Quadrant q = round(x*2/pi);
 * three-part Cody-Waite reduction r = x - q*pi/2 with pi/2 split as
 * 1.5703125 (8 significant bits, so q*C1 is exact) + 4.83826792e-4 +
 * 2.56334407e-12; then the Taylor series of sin to r^9 and cos to r^10 on
 * [-pi/4, pi/4] (truncation error below 1e-9).  Plain multiplies and adds
 * in a fixed order, so a CPU build without contraction and the GPU build
 * (-fmad=false) give identical bits. */
#define PT_SINCOS_BODY                                                          \
    float q = floorf(x * 0.636619747f + 0.5f);                                  \
    float r = ((x - q * 1.5703125f) - q * 4.83826792e-4f) - q * 2.56334407e-12f; \
    float r2 = r * r;                                                           \
    float sp = r + r * r2 * (-0.166666672f + r2 * (0.00833333377f +             \
               r2 * (-0.000198412701f + r2 * 2.75573188e-06f)));                \
    float cp = 1.f + r2 * (-0.5f + r2 * (0.0416666679f + r2 * (-0.00138888892f + \
               r2 * (2.48015876e-05f + r2 * -2.75573200e-07f))));               \
    int qi = ((int)q) & 3;                                                      \
    float sv = (qi == 0) ? sp : (qi == 1) ? cp : (qi == 2) ? -sp : -cp;          \
    float cv = (qi == 0) ? cp : (qi == 1) ? -sp : (qi == 2) ? -cp : sp;

static int g_portable_trig = 0;
void orc_set_portable_trig(int on) { g_portable_trig = on; }
static inline void orc_sincos(float x, float *s, float *c) {
    if (!g_portable_trig) { *s = sinf(x); *c = cosf(x); return; }
    PT_SINCOS_BODY
    *s = sv; *c = cv;
}

/* ------------------------------------------------------------------------- */
/* RNG: include/simplernd.h:35-49, rendering_kernel.cl:4-17                    */
/* ------------------------------------------------------------------------- */
float orc_get_random(uint32_t *seed0, uint32_t *seed1) {
    *seed0 = 36969u * ((*seed0) & 65535u) + ((*seed0) >> 16);
    *seed1 = 18000u * ((*seed1) & 65535u) + ((*seed1) >> 16);
    uint32_t ires = ((*seed0) << 16) + (*seed1);
    union { float f; uint32_t ui; } res;
    res.ui = (ires & 0x007fffffu) | 0x40000000u;
    return (res.f - 2.f) / 2.f;
}

uint64_t orc_splitmix64(uint64_t *state) {
    uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Seed array: replaces rand() clamped to >= 2 (smallptGPU.cpp:185-195). */
void orc_make_seeds(uint64_t master, uint32_t *seeds, uint32_t count) {
    uint64_t st = master;
    for (uint32_t i = 0; i < count; ++i) {
        uint32_t v = (uint32_t)orc_splitmix64(&st);
        seeds[i] = v < 2u ? 2u : v;
    }
}

/* ------------------------------------------------------------------------- */
/* camera: displayfunc.cpp:732-756, rendering_kernel.cl:1042-1070             */
/* ------------------------------------------------------------------------- */
void orc_update_camera(ptgpu_camera *cam) {
    float xd = sinf(cam->yaw) * cosf(cam->pitch);
    float yd = sinf(cam->pitch);
    float zd = cosf(cam->yaw) * cosf(cam->pitch);
    ptgpu_vec to_cam = v3(xd, yd, zd);
    cam->dir = vnorm(vsmul(-1.f, to_cam));
    const ptgpu_vec up = v3(0.f, 1.f, 0.f);
    const float fov = (ORC_PI / 180.f) * 45.f;
    cam->x = vnorm(vcross(cam->dir, up));
    cam->x = vsmul(cam->width * fov / cam->height, cam->x);
    cam->y = vnorm(vcross(cam->x, cam->dir));
    cam->y = vsmul(fov, cam->y);
}

void orc_generate_camera_ray(const ptgpu_camera *cam, uint32_t *s0, uint32_t *s1,
                             int w, int h, int x, int y, ptgpu_ray *ray) {
    const float inv_w = 1.f / (float)w;
    const float inv_h = 1.f / (float)h;
    const float r1 = orc_get_random(s0, s1) - .5f;
    const float r2 = orc_get_random(s0, s1) - .5f;
    const float kcx = ((float)x + r1) * inv_w - .5f;
    const float kcy = ((float)y + r2) * inv_h - .5f;
    ptgpu_vec rdir = v3(cam->x.x * kcx + cam->y.x * kcy + cam->dir.x,
                        cam->x.y * kcx + cam->y.y * kcy + cam->dir.y,
                        cam->x.z * kcx + cam->y.z * kcy + cam->dir.z);
    ptgpu_vec rorig = vadd(vsmul(0.1f, rdir), cam->orig);
    rdir = vnorm(rdir);
    ray->o = rorig;
    ray->d = rdir;
}

/* ------------------------------------------------------------------------- */
/* intersection: rendering_kernel.cl:26-56, 59-125 (non-TEST_CULL), 140-192   */
/* ------------------------------------------------------------------------- */
float orc_sphere_intersect(const ptgpu_sphere *s, const ptgpu_ray *r) {
    ptgpu_vec op = vsub(s->p, r->o);
    float b = vdot(op, r->d);
    float det = b * b - vdot(op, op) + s->rad * s->rad;
    if (det < 0.f) return 0.f;
    det = sqrtf(det);
    float t = b - det;
    if (t > ORC_EPSILON) return t;
    t = b + det;
    if (t > ORC_EPSILON) return t;
    return 0.f;
}

float orc_triangle_intersect(const ptgpu_triangle *tr, const ptgpu_ray *r) {
    ptgpu_vec e1 = vsub(tr->p2, tr->p1);
    ptgpu_vec e2 = vsub(tr->p3, tr->p1);
    ptgpu_vec pvec = vcross(r->d, e2);
    float det = vdot(e1, pvec);
    if (det == 0.f) return 0.f;
    /* 1.0/det in double then stored to float equals the float quotient:
     * double rounding is innocuous for division (53 >= 2*24+2). */
    float inv_det = 1.f / det;
    ptgpu_vec tvec = vsub(r->o, tr->p1);
    float u = vdot(tvec, pvec) * inv_det;
    if (u < 0.f || u > 1.f) return 0.f;
    ptgpu_vec qvec = vcross(tvec, e1);
    float v = vdot(r->d, qvec) * inv_det;
    if (v < 0.f || u + v > 1.f) return 0.f;
    float t = vdot(e2, qvec) * inv_det;
    if (t > ORC_EPSILON) return t;
    return 0.f;
}

int orc_bound_test(const ptgpu_ray *r, const ptgpu_bound *b) {
    float tmin, tmax;
    return orc_bound_test_t(r, b, &tmin, &tmax);
}

int orc_bound_test_t(const ptgpu_ray *r, const ptgpu_bound *b, float *tmin_out, float *tmax_out) {
    float xa = 1.f / r->d.x, ya = 1.f / r->d.y, za = 1.f / r->d.z;
    float xe = r->o.x, ye = r->o.y, ze = r->o.z;
    float txmin, txmax, tymin, tymax, tzmin, tzmax;
    if (xa >= 0) { txmin = (b->min_x - xe) * xa; txmax = (b->max_x - xe) * xa; }
    else         { txmin = (b->max_x - xe) * xa; txmax = (b->min_x - xe) * xa; }
    if (ya >= 0) { tymin = (b->min_y - ye) * ya; tymax = (b->max_y - ye) * ya; }
    else         { tymin = (b->max_y - ye) * ya; tymax = (b->min_y - ye) * ya; }
    if (za >= 0) { tzmin = (b->min_z - ze) * za; tzmax = (b->max_z - ze) * za; }
    else         { tzmin = (b->max_z - ze) * za; tzmax = (b->min_z - ze) * za; }
    float tmin = fmaxf(txmin, fmaxf(tymin, tzmin));
    float tmax = fminf(txmax, fminf(tymax, tzmax));
    *tmin_out = tmin;
    *tmax_out = tmax;
    return tmin <= tmax;
}

/* cull_closest: a box the walk may skip (see orc_accel) */
static inline int orc_box_enter(const orc_accel *acc, const ptgpu_ray *r, const ptgpu_bound *b,
                                float tbest) {
    float tmin, tmax;
    if (!orc_bound_test_t(r, b, &tmin, &tmax)) return 0;
    if (acc->cull_closest && (tmax < 0.f || tmin > tbest * 1.0001f)) return 0;
    return 1;
}

static inline float shape_intersect(const ptgpu_shape *s, const ptgpu_ray *r) {
    float d = 0.f;
    if (s->type == PTGPU_SPHERE) d = orc_sphere_intersect(&s->g.s, r);
    if (s->type == PTGPU_TRIANGLE) d = orc_triangle_intersect(&s->g.t, r);
    return d;
}

/* Intersect (rendering_kernel.cl:194-363).  The traversal stack is heap
 * allocated so deep trees are traced correctly (the reference's 18 entries
 * overflow beyond depth 17); everything else follows the reference order:
 * ACCELSTR 0 descending index, ACCELSTR 1/2 DFS left first, first found wins. */
#define ORC_STACK_MAX 256
int orc_intersect(const ptgpu_shape *shapes, uint32_t n, const orc_accel *acc,
                  const ptgpu_ray *r, float *t, uint32_t *id, orc_counters *cnt) {
    *t = ORC_INF_T;
    int accel = acc ? acc->accel : PTGPU_ACCEL_NONE;
    if (n == 0) return 0;
    if (accel == PTGPU_ACCEL_NONE || (accel == PTGPU_ACCEL_BVH && n == 1)) {
        for (uint32_t i = n; i--;) {
            float d = shape_intersect(&shapes[i], r);
            if (cnt) cnt->prim_tests++;
            if (d != 0.f && d < *t) { *t = d; *id = i; }
        }
        return *t < ORC_INF_T;
    }
    int intersected = 0;
    int32_t stack[ORC_STACK_MAX];
    int top = 0;
    if (accel == PTGPU_ACCEL_BVH) {
        /* items >= 0 are internal nodes, items < 0 are leaf -(k+1) */
        const ptgpu_bvh_node *btn = acc->btn, *btl = acc->btl;
        stack[top++] = 0;
        while (top > 0) {
            int32_t item = stack[--top];
            if (item < 0) {
                uint32_t sid = (uint32_t)btl[-item - 1].nShape;
                float d = shape_intersect(&shapes[sid], r);
                if (cnt) cnt->prim_tests++;
                if (d != 0.f) { if (d < *t) { *t = d; *id = sid; } intersected = 1; }
                continue;
            }
            const ptgpu_bvh_node *nd = &btn[item];
            if (cnt) cnt->node_visits++;
            if (!orc_box_enter(acc, r, &nd->bound, *t)) continue;
            int lleaf, rleaf;
            if (acc->bvh_reference_leafness) {
                lleaf = rleaf = (nd->leaf == 2);
                if (nd->leaf != 0 && nd->leaf != 2) continue;
            } else {
                lleaf = (nd->nLeft == nd->min);
                rleaf = (nd->nRight == nd->max);
            }
            if (top + 2 > ORC_STACK_MAX) return 0;
            stack[top++] = rleaf ? -(nd->nRight + 1) : nd->nRight;
            stack[top++] = lleaf ? -(nd->nLeft + 1) : nd->nLeft;
        }
        return intersected;
    }
    /* KD tree */
    stack[top++] = acc->kd_root;
    while (top > 0) {
        int32_t nidx = stack[--top];
        if (cnt) cnt->node_visits++;
        if (!orc_box_enter(acc, r, &acc->kd_box[nidx], *t)) continue;
        if (acc->kd_leaf[nidx] == 0) {
            if (acc->kd_left[nidx] < 0) continue; /* empty root (N == 0) */
            if (top + 2 > ORC_STACK_MAX) return 0;
            stack[top++] = acc->kd_right[nidx];
            stack[top++] = acc->kd_left[nidx];
        } else {
            for (int32_t i = acc->kd_min[nidx]; i < acc->kd_max[nidx]; i++) {
                uint32_t sid = (uint32_t)acc->kd_kn[i];
                float d = shape_intersect(&shapes[sid], r);
                if (cnt) cnt->prim_tests++;
                if (d != 0.f) { if (d < *t) { *t = d; *id = sid; } intersected = 1; }
            }
        }
    }
    return intersected;
}

/* IntersectP (rendering_kernel.cl:375-395): brute force over shapeCnt-2..0. */
int orc_intersect_p(const ptgpu_shape *shapes, uint32_t n, const ptgpu_ray *r, float maxt) {
    if (n == 0) return 0;
    uint32_t i = n - 1;
    for (; i--;) {
        float d = shape_intersect(&shapes[i], r);
        if (d != 0.f && d < maxt) return 1;
    }
    return 0;
}

/* IntersectP's predicate answered through the tree: a depth-first walk with
 * the reference's bound test (intersection_bound_test, no t culling, so it
 * enters every box the brute-force loop could find a hit in) that stops at
 * the first shape other than the last one with 0 < d < maxt.  An oracle-side
 * speed-up only: the reference tests every shape (rendering_kernel.cl:375-395). */
int orc_intersect_p_accel(const ptgpu_shape *shapes, uint32_t n, const orc_accel *acc,
                          const ptgpu_ray *r, float maxt) {
    if (!acc || !acc->shadow_accel || acc->accel == PTGPU_ACCEL_NONE ||
        (acc->accel == PTGPU_ACCEL_BVH && n <= 1))
        return orc_intersect_p(shapes, n, r, maxt);
    if (n <= 1) return 0;
    const uint32_t skip = n - 1;
    int32_t stack[ORC_STACK_MAX];
    int top = 0;
    if (acc->accel == PTGPU_ACCEL_BVH) {
        const ptgpu_bvh_node *btn = acc->btn, *btl = acc->btl;
        stack[top++] = 0;
        while (top > 0) {
            int32_t item = stack[--top];
            if (item < 0) {
                uint32_t sid = (uint32_t)btl[-item - 1].nShape;
                if (sid == skip) continue;
                float d = shape_intersect(&shapes[sid], r);
                if (d != 0.f && d < maxt) return 1;
                continue;
            }
            const ptgpu_bvh_node *nd = &btn[item];
            if (!orc_bound_test(r, &nd->bound)) continue;
            int lleaf = (nd->nLeft == nd->min), rleaf = (nd->nRight == nd->max);
            if (top + 2 > ORC_STACK_MAX) return orc_intersect_p(shapes, n, r, maxt);
            stack[top++] = rleaf ? -(nd->nRight + 1) : nd->nRight;
            stack[top++] = lleaf ? -(nd->nLeft + 1) : nd->nLeft;
        }
        return 0;
    }
    stack[top++] = acc->kd_root;
    while (top > 0) {
        int32_t nidx = stack[--top];
        if (!orc_bound_test(r, &acc->kd_box[nidx])) continue;
        if (acc->kd_leaf[nidx] == 0) {
            if (acc->kd_left[nidx] < 0) continue;
            if (top + 2 > ORC_STACK_MAX) return orc_intersect_p(shapes, n, r, maxt);
            stack[top++] = acc->kd_right[nidx];
            stack[top++] = acc->kd_left[nidx];
        } else {
            for (int32_t i = acc->kd_min[nidx]; i < acc->kd_max[nidx]; i++) {
                uint32_t sid = (uint32_t)acc->kd_kn[i];
                if (sid == skip) continue;
                float d = shape_intersect(&shapes[sid], r);
                if (d != 0.f && d < maxt) return 1;
            }
        }
    }
    return 0;
}

void orc_shadow_batch(const ptgpu_shape *shapes, uint32_t n, const orc_accel *acc,
                      const ptgpu_ray *rays, const float *maxt, uint32_t nrays,
                      int32_t *occluded, int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
    #pragma omp parallel for schedule(dynamic, 256) num_threads(threads)
#else
    (void)threads;
#endif
    for (int64_t i = 0; i < (int64_t)nrays; ++i)
        occluded[i] = (acc && acc->shadow_accel)
                          ? orc_intersect_p_accel(shapes, n, acc, &rays[i], maxt[i])
                          : orc_intersect_p(shapes, n, &rays[i], maxt[i]);
}

void orc_trace_closest(const ptgpu_shape *shapes, uint32_t n, const orc_accel *acc,
                       const ptgpu_ray *rays, uint32_t nrays, float *t,
                       uint32_t *id, int32_t *hit, orc_counters *cnt, int threads) {
    uint64_t visits = 0, tests = 0;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
    #pragma omp parallel for schedule(dynamic, 1024) num_threads(threads) reduction(+:visits, tests)
#else
    (void)threads;
#endif
    for (int64_t i = 0; i < (int64_t)nrays; ++i) {
        orc_counters c = {0, 0, 0};
        uint32_t rid = 0;
        float tt;
        int h = orc_intersect(shapes, n, acc, &rays[i], &tt, &rid, cnt ? &c : NULL);
        t[i] = tt; id[i] = h ? rid : 0u; hit[i] = h;
        visits += c.node_visits;
        tests += c.prim_tests;
    }
    if (cnt) {
        cnt->node_visits += visits;
        cnt->prim_tests += tests;
        cnt->rays += nrays;
    }
}

/* ------------------------------------------------------------------------- */
/* light sampling and shading: rendering_kernel.cl:127-135, 365-373, 397-493  */
/* ------------------------------------------------------------------------- */
static void two_randoms(uint32_t *s0, uint32_t *s1, int rtl, float *u1, float *u2) {
    if (rtl) { *u2 = orc_get_random(s0, s1); *u1 = orc_get_random(s0, s1); }
    else     { *u1 = orc_get_random(s0, s1); *u2 = orc_get_random(s0, s1); }
}

/* The emitters SampleLights visits: shapes with e != 0 in index order, until
 * lightCnt of them (rendering_kernel.cl:403-407).  Collected once per pass
 * instead of scanning the shape list at every diffuse hit; the order and the
 * set are the scan's.  Returns the count written to lights[]. */
static uint32_t collect_lights(const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt,
                               uint32_t *lights) {
    uint32_t i, visited;
    for (i = 0, visited = 0; i < n && visited < light_cnt; i++) {
        if (viszero(shapes[i].e)) continue;
        lights[visited++] = i;
    }
    return visited;
}

static void sample_lights(const ptgpu_shape *shapes, uint32_t n, const uint32_t *lights,
                          uint32_t n_lights, const orc_accel *acc,
                          int rtl, uint32_t *s0, uint32_t *s1, ptgpu_vec hit,
                          ptgpu_vec normal, ptgpu_vec *result) {
    *result = v3(0.f, 0.f, 0.f);
    for (uint32_t li = 0; li < n_lights; li++) {
        const ptgpu_shape *light = &shapes[lights[li]];
        ptgpu_ray shadow;
        shadow.o = hit;
        ptgpu_vec lp, ln;
        if (light->type == PTGPU_TRIANGLE) {
            float u1, u2;
            two_randoms(s0, s1, rtl, &u1, &u2);
            float su1 = sqrtf(u1);
            float bu = 1.0f - su1, bv = u2 * su1;
            ptgpu_vec e1 = vsub(light->g.t.p2, light->g.t.p1);
            ptgpu_vec e2 = vsub(light->g.t.p3, light->g.t.p1);
            e1 = vsmul(bu, e1);
            e2 = vsmul(bv, e2);
            lp = vadd(vadd(light->g.t.p1, e1), e2);
            ln = vnorm(vcross(e1, e2));
        } else {
            float u1, u2;
            two_randoms(s0, s1, rtl, &u1, &u2);
            const float zz = 1.f - 2.f * u1;
            const float rr = sqrtf(fmaxf(0.f, 1.f - zz * zz));
            const float phi = 2.f * ORC_PI * u2;
            float sphi, cphi;
            orc_sincos(phi, &sphi, &cphi);
            ptgpu_vec unit = v3(rr * cphi, rr * sphi, zz);
            lp = vadd(vsmul(light->g.s.rad, unit), light->g.s.p);
            ln = unit;
        }
        shadow.d = vsub(lp, hit);
        const float len = sqrtf(vdot(shadow.d, shadow.d));
        shadow.d = vsmul(1.f / len, shadow.d);
        float wo = vdot(shadow.d, ln);
        if (wo > 0.f) continue;
        wo = -wo;
        wo = cl_clamp(wo, 0.f, 1.f);
        const float wi = vdot(shadow.d, normal);
        if (wi > 0.f && !orc_intersect_p_accel(shapes, n, acc, &shadow, len - ORC_EPSILON)) {
            const float s = light->area * wi * wo / (len * len);
            *result = vadd(*result, vsmul(s, light->e));
        }
    }
}

/* Optional throughput Russian roulette, off by default (the reference has
 * none: its paths end only past MAX_DEPTH, rendering_kernel.cl:797-801).
 * With rr_depth = d > 0, a path about to continue past its hit at depth
 * `depth` >= d (and within max_depth) draws one random u and ends when
 * u >= p, p = min(max(throughput), 1); otherwise its throughput is divided by
 * p.  The GPU library's ptgpu_config.rr_depth does the same. */
static int g_rr_depth = 0;
void orc_set_rr_depth(int d) { g_rr_depth = d; }

/* 1: every diffuse hit scans the shape list for its emitters again, as the
 * reference's SampleLights does (rendering_kernel.cl:403-407,
 * geomfunc.h:383) -- the same lights in the same order, at the reference's
 * cost; for the timed CPU baseline.  0: the list collected once per pass. */
static int g_reference_cost = 0;
void orc_set_reference_cost(int on) { g_reference_cost = on; }
static int rr_stop(unsigned depth, int max_depth, ptgpu_vec *tp, uint32_t *s0, uint32_t *s1) {
    if (g_rr_depth <= 0 || (int)depth < g_rr_depth || (int)depth + 1 > max_depth) return 0;
    const float u = orc_get_random(s0, s1);
    const float p = fminf(fmaxf(tp->x, fmaxf(tp->y, tp->z)), 1.f);
    if (!(u < p)) return 1;
    *tp = vsmul(1.f / p, *tp);
    return 0;
}

/* RadianceOnePathTracing + RadiancePathTracing (rendering_kernel.cl:495-820) */
static void radiance(const ptgpu_shape *shapes, uint32_t n, const uint32_t *lights,
                     uint32_t n_lights, const orc_accel *acc, int max_depth, int rtl,
                     const ptgpu_ray *start, uint32_t *s0, uint32_t *s1, ptgpu_vec *result);

void orc_radiance(const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt,
                  const orc_accel *acc, int max_depth, int rtl,
                  const ptgpu_ray *start, uint32_t *s0, uint32_t *s1,
                  ptgpu_vec *result) {
    uint32_t cap = light_cnt < n ? light_cnt : n;
    uint32_t *lights = (uint32_t *)malloc(sizeof(uint32_t) * (cap ? cap : 1));
    uint32_t nl = collect_lights(shapes, n, light_cnt, lights);
    radiance(shapes, n, lights, nl, acc, max_depth, rtl, start, s0, s1, result);
    free(lights);
}

static void radiance(const ptgpu_shape *shapes, uint32_t n, const uint32_t *lights,
                     uint32_t n_lights, const orc_accel *acc, int max_depth, int rtl,
                     const ptgpu_ray *start, uint32_t *s0, uint32_t *s1, ptgpu_vec *result) {
    ptgpu_ray ray = *start;
    ptgpu_vec rad = v3(0.f, 0.f, 0.f);
    ptgpu_vec tp = v3(1.f, 1.f, 1.f);
    int specular = 1;
    for (unsigned depth = 0;; ++depth) {
        if (depth > (unsigned)max_depth) break;
        float t;
        uint32_t id = 0;
        if (!orc_intersect(shapes, n, acc, &ray, &t, &id, NULL)) break;
        ptgpu_vec hp = vadd(ray.o, vsmul(t, ray.d));
        const ptgpu_shape *s = &shapes[id];
        ptgpu_vec normal;
        if (s->type == PTGPU_SPHERE) normal = vsub(hp, s->g.s.p);
        else normal = vcross(vsub(s->g.t.p2, s->g.t.p1), vsub(s->g.t.p3, s->g.t.p1));
        normal = vnorm(normal);
        const float dp = vdot(normal, ray.d);
        const float inv_sign = -1.f * cl_sign(dp);
        ptgpu_vec nl = vsmul(inv_sign, normal);
        ptgpu_vec ecol = s->e;
        if (!viszero(ecol)) {
            if (specular) {
                ecol = vsmul(fabsf(dp), ecol);
                ecol = vmul(tp, ecol);
                rad = vadd(rad, ecol);
            }
            break;
        }
        ptgpu_vec col = s->c;
        if (s->refl == PTGPU_DIFF) {
            specular = 0;
            tp = vmul(tp, col);
            ptgpu_vec ld;
            if (g_reference_cost) {
                uint32_t again[8];
                if (n_lights <= 8 && collect_lights(shapes, n, n_lights, again) == n_lights)
                    sample_lights(shapes, n, again, n_lights, acc, rtl, s0, s1, hp, nl, &ld);
                else
                    sample_lights(shapes, n, lights, n_lights, acc, rtl, s0, s1, hp, nl, &ld);
            } else {
                sample_lights(shapes, n, lights, n_lights, acc, rtl, s0, s1, hp, nl, &ld);
            }
            ld = vmul(ld, tp);
            rad = vadd(rad, ld);
            float r1 = 2.f * ORC_PI * orc_get_random(s0, s1);
            float r2 = orc_get_random(s0, s1);
            float r2s = sqrtf(r2);
            ptgpu_vec w = nl;
            ptgpu_vec a = (fabsf(w.x) > .1f) ? v3(0.f, 1.f, 0.f) : v3(1.f, 0.f, 0.f);
            ptgpu_vec u = vnorm(vcross(a, w));
            ptgpu_vec v = vcross(w, u);
            float sr1, cr1;
            orc_sincos(r1, &sr1, &cr1);
            u = vsmul(cr1 * r2s, u);
            v = vsmul(sr1 * r2s, v);
            ptgpu_vec nd = vadd(u, v);
            w = vsmul(sqrtf(1.f - r2), w);
            nd = vadd(nd, w);
            ray.o = hp; ray.d = nd;
            if (rr_stop(depth, max_depth, &tp, s0, s1)) break;
        } else if (s->refl == PTGPU_SPEC) {
            specular = 1;
            ptgpu_vec nd = vsub(ray.d, vsmul(2.f * vdot(normal, ray.d), normal));
            tp = vmul(tp, col);
            ray.o = hp; ray.d = nd;
            if (rr_stop(depth, max_depth, &tp, s0, s1)) break;
        } else {
            specular = 1;
            ptgpu_vec refl_d = vsub(ray.d, vsmul(2.f * vdot(normal, ray.d), normal));
            int into = vdot(normal, nl) > 0;
            const float nc = 1.f, nt = 1.5f;
            float nnt = into ? nc / nt : nt / nc;
            float ddn = vdot(ray.d, nl);
            float cos2t = 1.f - nnt * nnt * (1.f - ddn * ddn);
            if (cos2t < 0.f) {
                tp = vmul(tp, col);
                ray.o = hp; ray.d = refl_d;
                if (rr_stop(depth, max_depth, &tp, s0, s1)) break;
                continue;
            }
            float kk = (float)(into ? 1 : -1) * (ddn * nnt + sqrtf(cos2t));
            ptgpu_vec nkk = vsmul(kk, normal);
            ptgpu_vec tdir = vnorm(vsub(vsmul(nnt, ray.d), nkk));
            float a = nt - nc, b = nt + nc;
            float R0 = a * a / (b * b);
            float c = 1.f - (into ? -ddn : vdot(tdir, normal));
            float Re = R0 + (1.f - R0) * c * c * c * c * c;
            float Tr = 1.f - Re;
            float P = .25f + .5f * Re;
            float RP = Re / P;
            float TP = Tr / (1.f - P);
            if (orc_get_random(s0, s1) < P) {
                tp = vsmul(RP, tp);
                tp = vmul(tp, col);
                ray.o = hp; ray.d = refl_d;
            } else {
                tp = vsmul(TP, tp);
                tp = vmul(tp, col);
                ray.o = hp; ray.d = tdir;
            }
            if (rr_stop(depth, max_depth, &tp, s0, s1)) break;
        }
    }
    *result = rad;
}

/* toInt (include/vec.h:60) */
uint32_t orc_to_int(float x) {
    return (uint32_t)(int)(powf(cl_clamp(x, 0.f, 1.f), 1.f / 2.2f) * 255.f + .5f);
}

/* RadianceGPU (rendering_kernel.cl:1072-1150) for rows [row_begin,row_end) */
void orc_render_pass(const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt,
                     const orc_accel *acc, int max_depth, int rtl,
                     const ptgpu_camera *cam, int w, int h, int current_sample,
                     ptgpu_vec *colors, uint32_t *pixels, uint32_t *seeds,
                     int row_begin, int row_end, int col_begin, int col_end, int threads) {
    if (row_end > h) row_end = h;
    if (col_end > w || col_end <= 0) col_end = w;
    if (col_begin < 0) col_begin = 0;
    uint32_t cap = light_cnt < n ? light_cnt : n;
    uint32_t *lights = (uint32_t *)malloc(sizeof(uint32_t) * (cap ? cap : 1));
    const uint32_t n_lights = collect_lights(shapes, n, light_cnt, lights);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
    /* pixels are independent (each has its own seed stream): rows and
     * columns are shared out together, so one row also uses every thread */
    #pragma omp parallel for collapse(2) schedule(dynamic, 8) num_threads(threads)
#else
    (void)threads;
#endif
    for (int y = row_begin; y < row_end; ++y) {
        for (int x = col_begin; x < col_end; ++x) {
            const int gid = y * w + x;
            uint32_t s0 = seeds[2 * gid], s1 = seeds[2 * gid + 1];
            ptgpu_ray ray;
            orc_generate_camera_ray(cam, &s0, &s1, w, h, x, y, &ray);
            ptgpu_vec r;
            radiance(shapes, n, lights, n_lights, acc, max_depth, rtl, &ray, &s0, &s1, &r);
            const int i = (h - y - 1) * w + x;
            if (current_sample == 0) {
                colors[i] = r;
            } else {
                const float k1 = (float)current_sample;
                const float k2 = 1.f / ((float)current_sample + 1.f);
                colors[i].x = (colors[i].x * k1 + r.x) * k2;
                colors[i].y = (colors[i].y * k1 + r.y) * k2;
                colors[i].z = (colors[i].z * k1 + r.z) * k2;
            }
            if (pixels)
                pixels[gid] = orc_to_int(colors[i].x) | (orc_to_int(colors[i].y) << 8) |
                              (orc_to_int(colors[i].z) << 16) | 0xff000000u;
            seeds[2 * gid] = s0;
            seeds[2 * gid + 1] = s1;
        }
    }
    free(lights);
}

/* ------------------------------------------------------------------------- */
/* LBVH                                                                       */
/* ------------------------------------------------------------------------- */
static ptgpu_bound shape_bound(const ptgpu_shape *s) {
    ptgpu_bound b;
    if (s->type == PTGPU_SPHERE) {          /* CLBVH.cpp:49-61 */
        const ptgpu_sphere *sp = &s->g.s;
        b.min_x = sp->p.x - sp->rad; b.max_x = sp->p.x + sp->rad;
        b.min_y = sp->p.y - sp->rad; b.max_y = sp->p.y + sp->rad;
        b.min_z = sp->p.z - sp->rad; b.max_z = sp->p.z + sp->rad;
    } else {                                 /* CLBVH.cpp:63-75 */
        const ptgpu_triangle *t = &s->g.t;
        b.min_x = min3f(t->p1.x, t->p2.x, t->p3.x); b.max_x = max3f(t->p1.x, t->p2.x, t->p3.x);
        b.min_y = min3f(t->p1.y, t->p2.y, t->p3.y); b.max_y = max3f(t->p1.y, t->p2.y, t->p3.y);
        b.min_z = min3f(t->p1.z, t->p2.z, t->p3.z); b.max_z = max3f(t->p1.z, t->p2.z, t->p3.z);
    }
    return b;
}

static uint32_t quantise10(float p, float lo, float hi) {
    /* (unsigned)(((p - min) / (max - min)) * CODE_OFFSET); NaN (max == min)
     * is defined as 0, values are in [0, 1024] otherwise. */
    float q = ((p - lo) / (hi - lo)) * 1024.f;
    if (!(q >= 0.f)) return 0u;
    if (q >= 4294967296.f) return 0u;
    return (uint32_t)q;
}

/* CLBVH::CLBVH bounds, centroid and Morton code (CLBVH.cpp:90-164) */
void orc_lbvh_morton(ptgpu_shape *shapes, uint32_t n) {
    float min_x = FLT_MAX, max_x = FLT_MIN;
    float min_y = FLT_MAX, max_y = FLT_MIN;
    float min_z = FLT_MAX, max_z = FLT_MIN;
    for (uint32_t i = 0; i < n; i++) {
        ptgpu_vec p;
        shapes[i].index = (int32_t)i;
        shapes[i].b = shape_bound(&shapes[i]);
        if (shapes[i].type == PTGPU_SPHERE) p = shapes[i].g.s.p;
        else p = v3((shapes[i].b.min_x + shapes[i].b.max_x) / 2.0f,
                    (shapes[i].b.min_y + shapes[i].b.max_y) / 2.0f,
                    (shapes[i].b.min_z + shapes[i].b.max_z) / 2.0f);
        if (p.x < min_x) min_x = p.x;
        if (p.x > max_x) max_x = p.x;
        if (p.y < min_y) min_y = p.y;
        if (p.y > max_y) max_y = p.y;
        if (p.z < min_z) min_z = p.z;
        if (p.z > max_z) max_z = p.z;
    }
    for (uint32_t i = 0; i < n; i++) {
        ptgpu_vec p;
        if (shapes[i].type == PTGPU_SPHERE) p = shapes[i].g.s.p;
        else {
            const ptgpu_triangle *t = &shapes[i].g.t;
            float lx = min3f(t->p1.x, t->p2.x, t->p3.x), hx = max3f(t->p1.x, t->p2.x, t->p3.x);
            float ly = min3f(t->p1.y, t->p2.y, t->p3.y), hy = max3f(t->p1.y, t->p2.y, t->p3.y);
            float lz = min3f(t->p1.z, t->p2.z, t->p3.z), hz = max3f(t->p1.z, t->p2.z, t->p3.z);
            p = v3((lx + hx) / 2.0f, (ly + hy) / 2.0f, (lz + hz) / 2.0f);
        }
        uint32_t a = quantise10(p.x, min_x, max_x);
        uint32_t b = quantise10(p.y, min_y, max_y);
        uint32_t c = quantise10(p.z, min_z, max_z);
        uint32_t code = 0;
        for (uint32_t j = 0; j < 10; j++) {
            code |= (((a >> (9 - j)) & 1u) << ((10 - j) * 3 - 1)) |
                    (((b >> (9 - j)) & 1u) << ((10 - j) * 3 - 2)) |
                    (((c >> (9 - j)) & 1u) << ((10 - j) * 3 - 3));
        }
        shapes[i].index = (int32_t)i;
        shapes[i].morton_code = code;
    }
}

/* CLBVH::bubblesort_Geometry (CLBVH.cpp:31-47): descending, stable. */
void orc_bubblesort_desc(const uint32_t *keys, uint32_t n, int32_t *sorted) {
    uint32_t *k = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) { k[i] = keys[i]; sorted[i] = (int32_t)i; }
    for (uint32_t level = 0; level + 1 < n; level++)
        for (uint32_t i = 0; i < n - level - 1; i++)
            if (k[i] < k[i + 1]) {
                uint32_t tk = k[i]; k[i] = k[i + 1]; k[i + 1] = tk;
                int32_t tv = sorted[i]; sorted[i] = sorted[i + 1]; sorted[i + 1] = tv;
            }
    free(k);
}

/* The same permutation in O(N): a stable LSD counting sort of ~key ascending
 * (a stable sort descending by key keeps equal keys in index order). */
void orc_sort_desc_stable(const uint32_t *keys, uint32_t n, int32_t *sorted) {
    int32_t *tmp = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) sorted[i] = (int32_t)i;
    for (int shift = 0; shift < 32; shift += 8) {
        uint32_t count[257];
        memset(count, 0, sizeof(count));
        for (uint32_t i = 0; i < n; i++) count[((~keys[sorted[i]]) >> shift & 255u) + 1]++;
        for (int d = 0; d < 256; d++) count[d + 1] += count[d];
        for (uint32_t i = 0; i < n; i++) tmp[count[(~keys[sorted[i]]) >> shift & 255u]++] = sorted[i];
        memcpy(sorted, tmp, sizeof(int32_t) * n);
    }
    free(tmp);
}

/* longestCommonPrefix on indices (BVH.cl:98-110, 127-134) */
static inline int lcp_idx(int i, int j, int len) {
    if (0 <= j && j < len) {
        uint32_t v = (uint32_t)(i ^ j);
        return v == 0 ? 32 : __builtin_clz(v);
    }
    return -1;
}

/* kernelConstructRadixTree (BVH.cl:141-208) for every internal node, with a
 * terminating search (the reference's split loop never reaches t = 0). */
void orc_radix_tree(uint32_t n, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl) {
    if (n >= 2) memset(btn, 0, sizeof(ptgpu_bvh_node) * (n - 1));
    memset(btl, 0xFF, sizeof(ptgpu_bvh_node) * n);
    const int len = (int)n;
    for (int i = 0; i + 1 < len; i++) {
        int d = (lcp_idx(i, i + 1, len) - lcp_idx(i, i - 1, len)) > 0 ? 1 : -1;
        int sig_min = lcp_idx(i, i - d, len);
        int lmax = 2;
        while (lcp_idx(i, i + lmax * d, len) > sig_min) lmax *= 2;
        int l = 0;
        for (int t = lmax / 2; t >= 1; t /= 2)
            if (lcp_idx(i, i + (l + t) * d, len) > sig_min) l += t;
        int j = i + l * d;
        int sig_node = lcp_idx(i, j, len);
        int s = 0;
        for (int div = 2;; div *= 2) {
            int t = (l + div - 1) / div;
            if (lcp_idx(i, i + (s + t) * d, len) > sig_node) s += t;
            if (t == 1) break;
        }
        int gamma = i + s * d + (d < 0 ? d : 0);
        ptgpu_bvh_node *cur = &btn[i];
        int lo = i < j ? i : j, hi = i < j ? j : i;
        cur->nLeft = gamma;
        cur->nRight = gamma + 1;
        if (lo == gamma) { cur->leaf = 2; btl[gamma].nParent = i; }
        else btn[gamma].nParent = i;
        if (hi == gamma + 1) { cur->leaf = 2; btl[gamma + 1].nParent = i; }
        else btn[gamma + 1].nParent = i;
        cur->min = lo;
        cur->max = hi;
    }
}

static ptgpu_bound merge_bounds(ptgpu_bound a, ptgpu_bound b) { /* BVH.cl:112-122 */
    ptgpu_bound c;
    c.min_x = min2f(a.min_x, b.min_x); c.max_x = max2f(a.max_x, b.max_x);
    c.min_y = min2f(a.min_y, b.min_y); c.max_y = max2f(a.max_y, b.max_y);
    c.min_z = min2f(a.min_z, b.min_z); c.max_z = max2f(a.max_z, b.max_z);
    return c;
}

/* kernelConstructBVHTree (BVH.cl:214-258) with its intent: leaves take the
 * sorted shape and its bound; each internal node is the union of its two real
 * children (child leafness from the node's range), computed bottom-up. */
static ptgpu_bound refit_node(int i, const ptgpu_bvh_node *btn_c, ptgpu_bvh_node *btn,
                              ptgpu_bvh_node *btl) {
    (void)btn_c;
    ptgpu_bvh_node *nd = &btn[i];
    ptgpu_bound lb = (nd->nLeft == nd->min) ? btl[nd->nLeft].bound : refit_node(nd->nLeft, btn_c, btn, btl);
    ptgpu_bound rb = (nd->nRight == nd->max) ? btl[nd->nRight].bound : refit_node(nd->nRight, btn_c, btn, btl);
    nd->bound = merge_bounds(lb, rb);
    return nd->bound;
}

void orc_refit(const ptgpu_shape *shapes, uint32_t n, const int32_t *sorted,
               ptgpu_bvh_node *btn, ptgpu_bvh_node *btl) {
    for (uint32_t k = 0; k < n; k++) {
        btl[k].bound = shapes[sorted[k]].b;
        btl[k].nShape = sorted[k];
    }
    if (n >= 2) refit_node(0, btn, btn, btl);
}

int orc_build_bvh(ptgpu_shape *shapes, uint32_t n, ptgpu_bvh_node *btn,
                  ptgpu_bvh_node *btl, int32_t *sorted) {
    if (n == 0) return PTGPU_E_INVAL;
    orc_lbvh_morton(shapes, n);
    uint32_t *keys = (uint32_t *)malloc(sizeof(uint32_t) * n);
    for (uint32_t i = 0; i < n; i++) keys[i] = shapes[i].morton_code;
    orc_sort_desc_stable(keys, n, sorted);
    free(keys);
    orc_radix_tree(n, btn, btl);
    orc_refit(shapes, n, sorted, btn, btl);
    return PTGPU_OK;
}

/* ------------------------------------------------------------------------- */
/* SAH cost and treelet restructuring (Karras & Aila, "Fast Parallel          */
/* Construction of High-Quality Bounding Volume Hierarchies", HPG 2013),      */
/* with the reference's constants Ci = 1.2, Ct = 1.0 (clheader.h:14-15) and   */
/* 7-leaf treelets (BVH.cl:400-471).                                          */
/* ------------------------------------------------------------------------- */
static float bound_area(const ptgpu_bound *b) {          /* BVH.cl:88-96 */
    float dx = b->max_x - b->min_x, dy = b->max_y - b->min_y, dz = b->max_z - b->min_z;
    return 2.f * (dx * dy + dx * dz + dy * dz);
}

/* SAH cost of the tree: Ci * sum(internal areas) + Ct * sum(leaf areas),
 * normalised by the root area. */
double orc_sah_cost(uint32_t n, const ptgpu_bvh_node *btn, const ptgpu_bvh_node *btl) {
    if (n < 2) return 1.0;
    double root = bound_area(&btn[0].bound), s = 0.0;
    for (uint32_t i = 0; i + 1 < n; i++) s += 1.2 * bound_area(&btn[i].bound);
    for (uint32_t i = 0; i < n; i++) s += 1.0 * bound_area(&btl[i].bound);
    return root > 0 ? s / root : s;
}

/* Node references inside the treelet code: >= 0 internal, < 0 leaf -(k+1). */
static int ref_is_leaf(int r) { return r < 0; }
static ptgpu_bound ref_bound(int r, const ptgpu_bvh_node *btn, const ptgpu_bvh_node *btl) {
    return r < 0 ? btl[-r - 1].bound : btn[r].bound;
}
static int child_ref(const ptgpu_bvh_node *nd, int right) {
    if (!right) return nd->nLeft == nd->min ? -(nd->nLeft + 1) : nd->nLeft;
    return nd->nRight == nd->max ? -(nd->nRight + 1) : nd->nRight;
}

static void treelet_at(int root, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl, float *cost,
                       const float *leaf_cost) {
    int leaves[7], nodes[6];
    int nl = 0, nn = 0;
    leaves[nl++] = child_ref(&btn[root], 0);
    leaves[nl++] = child_ref(&btn[root], 1);
    while (nl < 7) {                       /* expand the largest internal child */
        int best = -1; float best_a = -1.f;
        for (int i = 0; i < nl; i++) {
            if (ref_is_leaf(leaves[i])) continue;
            ptgpu_bound b = ref_bound(leaves[i], btn, btl);
            float a = bound_area(&b);
            if (a > best_a) { best_a = a; best = i; }
        }
        if (best < 0) break;
        int nd = leaves[best];
        nodes[nn++] = nd;
        leaves[best] = child_ref(&btn[nd], 0);
        leaves[nl++] = child_ref(&btn[nd], 1);
    }
    if (nl < 3) return;                    /* nothing to restructure */
    int nsub = 1 << nl;
    float area[128], copt[128];
    unsigned char popt[128];
    for (int s = 1; s < nsub; s++) {
        ptgpu_bound b = {FLT_MAX, -FLT_MAX, FLT_MAX, -FLT_MAX, FLT_MAX, -FLT_MAX};
        int first = 1;
        for (int i = 0; i < nl; i++) if (s >> i & 1) {
            ptgpu_bound c = ref_bound(leaves[i], btn, btl);
            b = first ? c : merge_bounds(b, c);
            first = 0;
        }
        area[s] = bound_area(&b);
    }
    for (int i = 0; i < nl; i++) {
        int r = leaves[i];
        copt[1 << i] = r < 0 ? leaf_cost[-r - 1] : cost[r];
    }
    for (int k = 2; k <= nl; k++) {
        for (int s = 1; s < nsub; s++) {
            if (__builtin_popcount((unsigned)s) != k) continue;
            float best = FLT_MAX; int bp = 0;
            int d = (s - 1) & s;
            int p = (-d) & s;
            while (p != 0) {
                float c = copt[p] + copt[s ^ p];
                if (c < best) { best = c; bp = p; }
                p = (p - d) & s;
            }
            copt[s] = 1.2f * area[s] + best;
            popt[s] = (unsigned char)bp;
        }
    }
    int full = nsub - 1;
    /* keep the original treelet unless the optimum is strictly cheaper */
    if (!(copt[full] < cost[root])) return;
    /* rebuild: internal node slots are root + nodes[], reused in DFS order */
    int slots[7]; int ns = 0;
    slots[ns++] = root;
    for (int i = 0; i < nn; i++) slots[ns++] = nodes[i];
    int used = 0;
    /* explicit stack of (subset, slot) */
    int st_s[16], st_n[16], top = 0;
    st_s[top] = full; st_n[top] = slots[used++]; top++;
    while (top) {
        top--;
        int s = st_s[top], nd = st_n[top];
        int ls = popt[s], rs = s ^ ls;
        int refs[2], subs[2] = {ls, rs};
        for (int c = 0; c < 2; c++) {
            if (__builtin_popcount((unsigned)subs[c]) == 1) {
                refs[c] = leaves[__builtin_ctz((unsigned)subs[c])];
            } else {
                refs[c] = slots[used++];
                st_s[top] = subs[c]; st_n[top] = refs[c]; top++;
            }
        }
        /* encode children in the BVHNodeGPU fields: leaf children are leaf
         * indices with min/max marking them, internal children node ids */
        ptgpu_bvh_node *p = &btn[nd];
        p->nLeft = refs[0] < 0 ? -refs[0] - 1 : refs[0];
        p->nRight = refs[1] < 0 ? -refs[1] - 1 : refs[1];
        p->min = refs[0] < 0 ? p->nLeft : -1;   /* min == nLeft marks a leaf  */
        p->max = refs[1] < 0 ? p->nRight : -1;  /* max == nRight marks a leaf */
        p->leaf = (refs[0] < 0 || refs[1] < 0) ? 2 : 0;
        if (refs[0] < 0) btl[-refs[0] - 1].nParent = nd; else btn[refs[0]].nParent = nd;
        if (refs[1] < 0) btl[-refs[1] - 1].nParent = nd; else btn[refs[1]].nParent = nd;
    }
    /* recompute bounds/costs of the rebuilt internal nodes bottom-up: the
     * slots were assigned top-down, so walk them in reverse */
    for (int i = used - 1; i >= 0; i--) {
        int nd = slots[i];
        ptgpu_bvh_node *p = &btn[nd];
        int lr = p->min == p->nLeft ? -(p->nLeft + 1) : p->nLeft;
        int rr = p->max == p->nRight ? -(p->nRight + 1) : p->nRight;
        ptgpu_bound lb = ref_bound(lr, btn, btl), rb = ref_bound(rr, btn, btl);
        p->bound = merge_bounds(lb, rb);
        float lc = lr < 0 ? leaf_cost[-lr - 1] : cost[lr];
        float rc = rr < 0 ? leaf_cost[-rr - 1] : cost[rr];
        cost[nd] = 1.2f * bound_area(&p->bound) + lc + rc;
    }
}

static void treelet_rec(int nd, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl, float *cost,
                        const float *leaf_cost) {
    ptgpu_bvh_node *p = &btn[nd];
    int lr = p->min == p->nLeft ? -(p->nLeft + 1) : p->nLeft;
    int rr = p->max == p->nRight ? -(p->nRight + 1) : p->nRight;
    if (lr >= 0) treelet_rec(lr, btn, btl, cost, leaf_cost);
    if (rr >= 0) treelet_rec(rr, btn, btl, cost, leaf_cost);
    float lc = lr < 0 ? leaf_cost[-lr - 1] : cost[lr];
    float rc = rr < 0 ? leaf_cost[-rr - 1] : cost[rr];
    cost[nd] = 1.2f * bound_area(&p->bound) + lc + rc;
    treelet_at(nd, btn, btl, cost, leaf_cost);
}

/* Sequential bottom-up treelet passes (`sweeps` of them, each over the tree
 * the previous one left).  After them, internal nodes mark leaf children with
 * min == nLeft / max == nRight and internal children with -1 in min/max;
 * leaf==2 still flags "has a leaf child". */
int orc_treelet_optimize_sweeps(uint32_t n, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl, int sweeps) {
    if (n < 3) return PTGPU_OK;
    float *cost = (float *)calloc(n, sizeof(float));
    float *leaf_cost = (float *)calloc(n, sizeof(float));
    for (uint32_t k = 0; k < n; k++) leaf_cost[k] = 1.0f * bound_area(&btl[k].bound);
    /* normalise the child encoding to the min/max marking first */
    for (uint32_t i = 0; i + 1 < n; i++) {
        ptgpu_bvh_node *p = &btn[i];
        int lleaf = p->nLeft == p->min, rleaf = p->nRight == p->max;
        p->min = lleaf ? p->nLeft : -1;
        p->max = rleaf ? p->nRight : -1;
    }
    for (int it = 0; it < sweeps; it++) treelet_rec(0, btn, btl, cost, leaf_cost);
    for (uint32_t i = 0; i + 1 < n; i++) { btn[i].cost = cost[i]; btn[i].area = bound_area(&btn[i].bound); }
    free(cost); free(leaf_cost);
    return PTGPU_OK;
}

int orc_treelet_optimize(uint32_t n, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl) {
    return orc_treelet_optimize_sweeps(n, btn, btl, 1);
}

/* ------------------------------------------------------------------------- */
/* KD tree: KDTree.cpp:46-182 (build), 184-270 (heap export)                  */
/* ------------------------------------------------------------------------- */
static ptgpu_vec kd_midpoint(const ptgpu_shape *s) {
    if (s->type == PTGPU_TRIANGLE) {
        /* (t.p1.x, t.p2.x, t.p3.x) / 3.0f is a comma expression: p3 / 3 */
        return v3(s->g.t.p3.x / 3.0f, s->g.t.p3.y / 3.0f, s->g.t.p3.z / 3.0f);
    }
    return s->g.s.p;
}

static void kd_expand(ptgpu_bound *box, ptgpu_bound b) {      /* KDTree.h:35-44 */
    if (b.min_x < box->min_x) box->min_x = b.min_x;
    if (b.min_y < box->min_y) box->min_y = b.min_y;
    if (b.min_z < box->min_z) box->min_z = b.min_z;
    if (b.max_x > box->max_x) box->max_x = b.max_x;
    if (b.max_y > box->max_y) box->max_y = b.max_y;
    if (b.max_z > box->max_z) box->max_z = b.max_z;
}

static int kd_longest_axis(ptgpu_bound b) {                    /* KDTree.cpp:72-86 */
    float xd = b.max_x - b.min_x, yd = b.max_y - b.min_y, zd = b.max_z - b.min_z;
    if (xd >= yd) return xd >= zd ? 0 : 2;
    return yd >= zd ? 1 : 2;
}

static int kd_new_node(orc_kdtree *kd) {
    if (kd->n_nodes == kd->cap_nodes) {
        int cap = kd->cap_nodes ? kd->cap_nodes * 2 : 1024;
        kd->leaf = (int32_t *)realloc(kd->leaf, sizeof(int32_t) * cap);
        kd->left = (int32_t *)realloc(kd->left, sizeof(int32_t) * cap);
        kd->right = (int32_t *)realloc(kd->right, sizeof(int32_t) * cap);
        kd->depth = (int32_t *)realloc(kd->depth, sizeof(int32_t) * cap);
        kd->kmin = (int32_t *)realloc(kd->kmin, sizeof(int32_t) * cap);
        kd->kmax = (int32_t *)realloc(kd->kmax, sizeof(int32_t) * cap);
        kd->box = (ptgpu_bound *)realloc(kd->box, sizeof(ptgpu_bound) * cap);
        kd->cap_nodes = cap;
    }
    int id = kd->n_nodes++;
    kd->leaf[id] = 0; kd->left[id] = -1; kd->right[id] = -1;
    kd->kmin[id] = 0; kd->kmax[id] = 0;
    memset(&kd->box[id], 0, sizeof(ptgpu_bound));
    return id;
}

/* leaf shape lists are kept per node in a side table until export */
typedef struct { int32_t *ids; int32_t cnt; } kd_list;

static int kd_build_rec(const ptgpu_shape *shapes, int32_t *ids, int32_t cnt, int depth,
                        orc_kdtree *kd, kd_list **lists, int *lists_cap) {
    int node = kd_new_node(kd);
    if (node >= *lists_cap) {
        int cap = *lists_cap ? *lists_cap * 2 : 1024;
        while (cap <= node) cap *= 2;
        *lists = (kd_list *)realloc(*lists, sizeof(kd_list) * cap);
        *lists_cap = cap;
    }
    (*lists)[node].ids = NULL; (*lists)[node].cnt = 0;
    kd->depth[node] = depth;
    if (depth > kd->max_depth) kd->max_depth = depth;
    if (cnt == 0) return node;
    if (cnt <= 1) {
        kd->leaf[node] = 1;
        kd->box[node] = shape_bound(&shapes[ids[0]]);
        (*lists)[node].ids = (int32_t *)malloc(sizeof(int32_t));
        (*lists)[node].ids[0] = ids[0]; (*lists)[node].cnt = 1;
        kd->szbuf += cnt;
        return node;
    }
    ptgpu_vec mid = v3(0.f, 0.f, 0.f);
    float recp = (float)(1.0 / (double)cnt);
    ptgpu_bound box = shape_bound(&shapes[ids[0]]);
    for (int32_t i = 1; i < cnt; i++) {
        kd_expand(&box, shape_bound(&shapes[ids[i]]));
        ptgpu_vec m = kd_midpoint(&shapes[ids[i]]);
        m.x *= recp; m.y *= recp; m.z *= recp;
        mid.x += m.x; mid.y += m.y; mid.z += m.z;
    }
    kd->box[node] = box;
    int axis = kd_longest_axis(box);
    int32_t *lft = (int32_t *)malloc(sizeof(int32_t) * cnt);
    int32_t *rgt = (int32_t *)malloc(sizeof(int32_t) * cnt);
    int32_t nl = 0, nr = 0;
    for (int32_t i = 0; i < cnt; i++) {
        ptgpu_vec m = kd_midpoint(&shapes[ids[i]]);
        float mv = axis == 0 ? m.x : (axis == 1 ? m.y : m.z);
        float cv = axis == 0 ? mid.x : (axis == 1 ? mid.y : mid.z);
        if (cv >= mv) rgt[nr++] = ids[i]; else lft[nl++] = ids[i];
    }
    if (nl == cnt || nr == cnt) {
        kd->leaf[node] = 1;
        (*lists)[node].ids = (int32_t *)malloc(sizeof(int32_t) * cnt);
        memcpy((*lists)[node].ids, ids, sizeof(int32_t) * cnt);
        (*lists)[node].cnt = cnt;
        kd->szbuf += cnt;
        free(lft); free(rgt);
        return node;
    }
    int l = kd_build_rec(shapes, lft, nl, depth + 1, kd, lists, lists_cap);
    free(lft);
    int r = kd_build_rec(shapes, rgt, nr, depth + 1, kd, lists, lists_cap);
    free(rgt);
    kd->left[node] = l;
    kd->right[node] = r;
    return node;
}

/* Builds the pointer tree; kn is filled in BFS order (traverseTree order). */
int orc_kd_build(const ptgpu_shape *shapes, uint32_t n, orc_kdtree *out) {
    memset(out, 0, sizeof(*out));
    int32_t *ids = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) ids[i] = (int32_t)i;
    kd_list *lists = NULL; int lists_cap = 0;
    kd_build_rec(shapes, ids, (int32_t)n, 0, out, &lists, &lists_cap);
    free(ids);
    out->kn = (int32_t *)malloc(sizeof(int32_t) * (out->szbuf ? out->szbuf : 1));
    out->kn_cap = out->szbuf;
    /* BFS over real nodes: the heap BFS with null placeholders visits the
     * real nodes in the same order. */
    int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * out->n_nodes);
    int qh = 0, qt = 0;
    queue[qt++] = 0;
    while (qh < qt) {
        int nd = queue[qh++];
        if (out->leaf[nd]) {
            out->kmin[nd] = out->kn_cnt;
            for (int32_t i = 0; i < lists[nd].cnt; i++) out->kn[out->kn_cnt++] = lists[nd].ids[i];
            out->kmax[nd] = out->kn_cnt;
        }
        if (out->left[nd] >= 0) queue[qt++] = out->left[nd];
        if (out->right[nd] >= 0) queue[qt++] = out->right[nd];
    }
    free(queue);
    for (int i = 0; i < out->n_nodes; i++) free(lists[i].ids);
    free(lists);
    return PTGPU_OK;
}

void orc_kd_free(orc_kdtree *kd) {
    free(kd->leaf); free(kd->left); free(kd->right); free(kd->depth);
    free(kd->kmin); free(kd->kmax); free(kd->box); free(kd->kn);
    memset(kd, 0, sizeof(*kd));
}

int orc_kd_heap(const orc_kdtree *kd, ptgpu_kd_node *kng, int32_t kng_cnt, int32_t *kn) {
    int64_t size = (int64_t)1 << (kd->max_depth + 1);
    if (kng_cnt < size) return PTGPU_E_INVAL;
    memset(kng, 0, sizeof(ptgpu_kd_node) * (size_t)size);
    int range_ok = size <= 32768 && kd->szbuf <= 32767;
    /* heap position of each real node: root 1, children 2p and 2p+1 */
    int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * (kd->n_nodes ? kd->n_nodes : 1));
    int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * (kd->n_nodes ? kd->n_nodes : 1));
    int qh = 0, qt = 0;
    if (kd->n_nodes) { queue[qt++] = 0; pos[0] = 1; }
    while (qh < qt) {
        int nd = queue[qh++];
        int64_t p = pos[nd];
        ptgpu_kd_node *k = &kng[p];
        k->bound = kd->box[nd];
        k->leaf = (int16_t)kd->leaf[nd];
        if (kd->leaf[nd]) { k->min = (int16_t)kd->kmin[nd]; k->max = (int16_t)kd->kmax[nd]; }
        k->nLeft = (int16_t)(2 * p);
        k->nRight = (int16_t)(2 * p + 1);
        k->nParent = (int16_t)(p / 2);
        if (kd->left[nd] >= 0) { pos[kd->left[nd]] = 2 * p; queue[qt++] = kd->left[nd]; }
        if (kd->right[nd] >= 0) { pos[kd->right[nd]] = 2 * p + 1; queue[qt++] = kd->right[nd]; }
    }
    free(pos); free(queue);
    memcpy(kn, kd->kn, sizeof(int32_t) * (size_t)kd->kn_cnt);
    return range_ok ? PTGPU_OK : PTGPU_E_RANGE;
}
