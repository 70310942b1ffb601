/*
 * ptgpu_oracle.h -- CPU oracle for the PTGPU_PC hot path (TEST INFRASTRUCTURE).
 *
 * This is a plain-C restatement of the reference algorithms, used only as the
 * checker by the test suite, by the smoke check and as the timed CPU baseline.
 * It is never linked into, called by, or shipped with the GPU library.
 * Each function cites the reference file:line it restates.
 */
#ifndef PTGPU_ORACLE_H
#define PTGPU_ORACLE_H

#include "../include/ptgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Counters for the algorithmic-bytes model: bound tests and primitive tests. */
typedef struct {
    uint64_t node_visits;
    uint64_t prim_tests;
    uint64_t rays;
} orc_counters;

/* accel structure view used by the tracing functions */
typedef struct {
    int32_t accel;                   /* PTGPU_ACCEL_*                       */
    const ptgpu_bvh_node *btn, *btl; /* BVH (accel 1)                       */
    int32_t bvh_reference_leafness;  /* 1: leaf==2 => both children leaves  */
    const int32_t *kd_leaf, *kd_left, *kd_right; /* KD pointer tree (accel 2) */
    const ptgpu_bound *kd_box;
    const int32_t *kd_min, *kd_max;  /* leaf ranges into kd_kn              */
    const int32_t *kd_kn;
    int32_t kd_root;
    /* 0: shadow rays by the reference's brute-force IntersectP; 1: the same
     * predicate (any shape but the last with 0 < d < maxt) answered through
     * the BVH or KD tree above, for scenes where brute force is too slow on
     * the CPU.  The two are compared on the CPU by the test suite. */
    int32_t shadow_accel;
    /* 1: the closest-hit walk (BVH/KD) skips a box whose entry distance is
     * beyond the best hit so far by more than rounding (1e-4 relative) or whose
     * exit lies behind the origin.  No box it skips can hold a hit the walk
     * would keep, and the visit order is unchanged, so results are the
     * reference walk's; another oracle-side speed-up, compared on the CPU by
     * the test suite. */
    int32_t cull_closest;
} orc_accel;

/* RNG and camera */
float orc_get_random(uint32_t *seed0, uint32_t *seed1);
void  orc_update_camera(ptgpu_camera *cam);
void  orc_generate_camera_ray(const ptgpu_camera *cam, uint32_t *s0, uint32_t *s1,
                              int w, int h, int x, int y, ptgpu_ray *ray);
uint64_t orc_splitmix64(uint64_t *state);
void  orc_make_seeds(uint64_t master, uint32_t *seeds, uint32_t count);

/* intersection */
float orc_sphere_intersect(const ptgpu_sphere *s, const ptgpu_ray *r);
float orc_triangle_intersect(const ptgpu_triangle *tr, const ptgpu_ray *r);
int   orc_bound_test(const ptgpu_ray *r, const ptgpu_bound *b);
/* the same test, also returning the entry and exit distances */
int   orc_bound_test_t(const ptgpu_ray *r, const ptgpu_bound *b, float *tmin, float *tmax);
int   orc_intersect(const ptgpu_shape *shapes, uint32_t n, const orc_accel *acc,
                    const ptgpu_ray *r, float *t, uint32_t *id, orc_counters *cnt);
int   orc_intersect_p(const ptgpu_shape *shapes, uint32_t n, const ptgpu_ray *r,
                      float maxt);
int   orc_intersect_p_accel(const ptgpu_shape *shapes, uint32_t n, const orc_accel *acc,
                            const ptgpu_ray *r, float maxt);
/* one shadow query per ray (maxt[i]); occluded[i] = 1 when any shape but the
 * last is hit at 0 < d < maxt[i]; accel == NULL or shadow_accel == 0: brute
 * force */
void  orc_shadow_batch(const ptgpu_shape *shapes, uint32_t n, const orc_accel *acc,
                       const ptgpu_ray *rays, const float *maxt, uint32_t nrays,
                       int32_t *occluded, int threads);
void  orc_trace_closest(const ptgpu_shape *shapes, uint32_t n, const orc_accel *acc,
                        const ptgpu_ray *rays, uint32_t nrays, float *t,
                        uint32_t *id, int32_t *hit, orc_counters *cnt, int threads);

/* path tracing (arg_order_rtl = 1 evaluates the two random arguments of the
 * light samplers right-to-left, which is what g++ does with the reference
 * source; 0 is left-to-right, the OpenCL/clang order the GPU follows) */
void  orc_radiance(const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt,
                   const orc_accel *acc, int max_depth, int arg_order_rtl,
                   const ptgpu_ray *start, uint32_t *s0, uint32_t *s1,
                   ptgpu_vec *result);
void  orc_render_pass(const ptgpu_shape *shapes, uint32_t n, uint32_t light_cnt,
                      const orc_accel *acc, int max_depth, int arg_order_rtl,
                      const ptgpu_camera *cam, int w, int h, int current_sample,
                      ptgpu_vec *colors, uint32_t *pixels, uint32_t *seeds,
                      int row_begin, int row_end, int col_begin, int col_end, int threads);
uint32_t orc_to_int(float x);
/* 0: sin/cos from libm (as the reference source compiled here); 1: the
 * library's own deterministic sin/cos (as the GPU computes them) */
void  orc_set_portable_trig(int on);
/* 0: no throughput Russian roulette (the reference); d > 0: roulette from
 * the hit at depth d on (see rr_stop in ptgpu_oracle.c) */
void  orc_set_rr_depth(int d);
/* 1: SampleLights rescans the shapes for emitters at every diffuse hit, as
 * the reference does (the timed CPU baseline); 0: once per pass */
void  orc_set_reference_cost(int on);

/* LBVH */
void  orc_lbvh_morton(ptgpu_shape *shapes, uint32_t n);
void  orc_sort_desc_stable(const uint32_t *keys, uint32_t n, int32_t *sorted);
void  orc_bubblesort_desc(const uint32_t *keys, uint32_t n, int32_t *sorted);
void  orc_radix_tree(uint32_t n, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl);
void  orc_refit(const ptgpu_shape *shapes, uint32_t n, const int32_t *sorted,
                ptgpu_bvh_node *btn, ptgpu_bvh_node *btl);
int   orc_build_bvh(ptgpu_shape *shapes, uint32_t n, ptgpu_bvh_node *btn,
                    ptgpu_bvh_node *btl, int32_t *sorted);
double orc_sah_cost(uint32_t n, const ptgpu_bvh_node *btn, const ptgpu_bvh_node *btl);
int   orc_treelet_optimize(uint32_t n, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl);
int   orc_treelet_optimize_sweeps(uint32_t n, ptgpu_bvh_node *btn, ptgpu_bvh_node *btl, int sweeps);

/* KD tree (pointer tree arrays, nodes numbered in creation order, root 0) */
typedef struct {
    int32_t n_nodes, cap_nodes;
    int32_t *leaf, *left, *right, *depth;
    ptgpu_bound *box;
    int32_t *kmin, *kmax;     /* range into kn (leaves), filled in BFS order */
    int32_t *kn; int32_t kn_cnt, kn_cap;
    int32_t max_depth;
    int32_t szbuf;
} orc_kdtree;
int   orc_kd_build(const ptgpu_shape *shapes, uint32_t n, orc_kdtree *out);
void  orc_kd_free(orc_kdtree *kd);
/* KDTree::getTrees heap export; returns 0 or PTGPU_E_RANGE (int16 overflow).
 * kng must hold 2^(max_depth+1) nodes; null slots are zeroed. */
int   orc_kd_heap(const orc_kdtree *kd, ptgpu_kd_node *kng, int32_t kng_cnt,
                  int32_t *kn);

#ifdef __cplusplus
}
#endif
#endif
