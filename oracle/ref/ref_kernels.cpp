/*
 * ref_kernels.cpp -- compiles the reference's OpenCL kernels (BVH.cl and
 * rendering_kernel.cl at ACCELSTR 0, 1 and 2) as host C++ and exposes them
 * through a C ABI, so the oracle restatement can be checked against the
 * reference's own code.  TEST INFRASTRUCTURE ONLY: built by oracle/ref/build_ref.sh
 * into oracle/_ref/, never part of the GPU library.
 *
 * The OpenCL C built-ins the kernels use get their OpenCL meaning:
 * max/min = fmax/fmin, clamp = fmin(fmax(x, lo), hi), sign(0) = 0,
 * atomic_add = fetch-and-add (the NDRange runs sequentially), get_global_id
 * returns the emulated work-item id.
 */
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "cl_stub.h"

/* ---- OpenCL C shim -------------------------------------------------------- */
#define GPU_KERNEL 1
#define __kernel
#define __global
#define __constant
#define __local
static thread_local int ref_gid = 0;
static inline int get_global_id(int) { return ref_gid; }
static inline float max(float a, float b) { return std::fmax(a, b); }
static inline float min(float a, float b) { return std::fmin(a, b); }
static inline float clamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
static inline float sign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : (x == x ? x : 0.f)); }
static inline int atomic_add(int *p, int v) { int o = *p; *p += v; return o; }
using std::sqrt; using std::sin; using std::cos; using std::pow; using std::fabs;

/* shared types, then the kernels in their own namespaces */
#include "include/clheader.h"

namespace bvhcl {
#include "BVH.cl"   /* oracle/_ref/gen/BVH.cl: the reference file with the split-loop guard */
}

#undef ACCELSTR
#define ACCELSTR 0
namespace rk0 {
#include "include/rendering_kernel.cl"
}
#undef ACCELSTR
#define ACCELSTR 1
namespace rk1 {
#include "include/rendering_kernel.cl"
}
#undef ACCELSTR
#define ACCELSTR 2
namespace rk2 {
#include "include/rendering_kernel.cl"
}

/* ---- OpenCL host API emulation used by CLBVH.cpp --------------------------- */
struct ref_cl_mem_s { std::vector<unsigned char> data; };
struct ref_cl_kernel_s {
    int which;                      /* 0 radix tree, 1 BVH refit, 2 optimise */
    std::vector<std::vector<unsigned char>> args;
};

extern "C" cl_kernel ref_make_kernel(int which) {
    cl_kernel k = new ref_cl_kernel_s();
    k->which = which;
    k->args.resize(8);
    return k;
}
extern "C" void ref_free_kernel(cl_kernel k) { delete k; }

cl_mem clCreateBuffer(cl_context, cl_mem_flags, size_t size, void *, cl_int *st) {
    cl_mem m = new ref_cl_mem_s();
    m->data.resize(size ? size : 1);
    if (st) *st = CL_SUCCESS;
    return m;
}
cl_int clReleaseMemObject(cl_mem m) { delete m; return CL_SUCCESS; }
cl_int clEnqueueWriteBuffer(cl_command_queue, cl_mem m, cl_bool, size_t off, size_t sz,
                            const void *p, cl_uint, const cl_event *, cl_event *) {
    if (sz) std::memcpy(m->data.data() + off, p, sz);
    return CL_SUCCESS;
}
cl_int clEnqueueReadBuffer(cl_command_queue, cl_mem m, cl_bool, size_t off, size_t sz,
                           void *p, cl_uint, const cl_event *, cl_event *) {
    if (sz) std::memcpy(p, m->data.data() + off, sz);
    return CL_SUCCESS;
}
cl_int clSetKernelArg(cl_kernel k, cl_uint idx, size_t sz, const void *v) {
    if (idx >= k->args.size()) k->args.resize(idx + 1);
    k->args[idx].assign((const unsigned char *)v, (const unsigned char *)v + sz);
    return CL_SUCCESS;
}
cl_int clFinish(cl_command_queue) { return CL_SUCCESS; }

template <typename T> static T arg_val(cl_kernel k, int i) {
    T v; std::memcpy(&v, k->args[i].data(), sizeof(T)); return v;
}
template <typename T> static T *arg_buf(cl_kernel k, int i) {
    cl_mem m = arg_val<cl_mem>(k, i);
    return reinterpret_cast<T *>(m->data.data());
}

cl_int clEnqueueNDRangeKernel(cl_command_queue, cl_kernel k, cl_uint, const size_t *,
                              const size_t *global, const size_t *, cl_uint,
                              const cl_event *, cl_event *) {
    for (size_t g = 0; g < global[0]; ++g) {
        ref_gid = (int)g;
        switch (k->which) {
        case 0:
            bvhcl::kernelConstructRadixTree(arg_val<int>(k, 0), arg_buf<BVHNodeGPU>(k, 1),
                                            arg_buf<BVHNodeGPU>(k, 2));
            break;
        case 1:
            bvhcl::kernelConstructBVHTree(arg_buf<Shape>(k, 0), arg_val<int>(k, 1),
                                          arg_buf<BVHNodeGPU>(k, 2), arg_buf<BVHNodeGPU>(k, 3),
                                          arg_buf<int>(k, 4), arg_buf<int>(k, 5));
            break;
        default:
            break;
        }
    }
    return CL_SUCCESS;
}

/* ---- C ABI over the kernels ------------------------------------------------ */
extern "C" {

float ref_get_random(unsigned int *s0, unsigned int *s1) { return rk0::GetRandom(s0, s1); }

/* kernelConstructRadixTree over N-1 work-items with the CLBVH buffer init */
void ref_radix_tree(int n, BVHNodeGPU *btn, BVHNodeGPU *btl) {
    if (n >= 2) std::memset(btn, 0, sizeof(BVHNodeGPU) * (n - 1));
    std::memset(btl, 0xFF, sizeof(BVHNodeGPU) * n);
    int internal = n - 1;
    for (int g = 0; g < internal; ++g) {
        ref_gid = g;
        bvhcl::kernelConstructRadixTree(internal, btn, btl);
    }
}

/* one RadianceGPU NDRange (all W*H work-items) for the given ACCELSTR */
void ref_render_pass(int accel, Vec *colors, unsigned int *seeds, Camera *cam,
                     Shape *shapes, unsigned int n, unsigned int light_cnt,
                     BVHNodeGPU *btn, BVHNodeGPU *btl, KDNodeGPU *kng, int kng_cnt,
                     int *kn, int kn_cnt, int w, int h, int current_sample,
                     int *pixels) {
    for (int g = 0; g < w * h; ++g) {
        ref_gid = g;
        if (accel == 0)
            rk0::RadianceGPU(colors, seeds, cam, shapes, n, light_cnt, w, h, current_sample, pixels);
        else if (accel == 1)
            rk1::RadianceGPU(colors, seeds, cam, shapes, n, light_cnt, btn, btl, w, h,
                             current_sample, pixels);
        else
            rk2::RadianceGPU(colors, seeds, cam, shapes, n, light_cnt, kng, kng_cnt, kn, kn_cnt,
                             w, h, current_sample, pixels);
    }
}

/* Intersect for a batch of rays */
void ref_intersect(int accel, Shape *shapes, unsigned int n, BVHNodeGPU *btn,
                   BVHNodeGPU *btl, KDNodeGPU *kng, int kng_cnt, int *kn, int kn_cnt,
                   const Ray *rays, int nrays, float *t, unsigned int *id, int *hit) {
    for (int i = 0; i < nrays; ++i) {
        ref_gid = i;
        float tt = 0.f;
        unsigned int rid = 0;
        int h;
        if (accel == 0) h = rk0::Intersect(shapes, n, &rays[i], &tt, &rid);
        else if (accel == 1) h = rk1::Intersect(shapes, n, btn, btl, &rays[i], &tt, &rid);
        else h = rk2::Intersect(shapes, n, kng, kng_cnt, kn, kn_cnt, &rays[i], &tt, &rid);
        t[i] = tt; id[i] = h ? rid : 0u; hit[i] = h;
    }
}

int ref_intersect_p(Shape *shapes, unsigned int n, const Ray *r, float maxt) {
    return rk0::IntersectP(shapes, n, r, maxt);
}

void ref_generate_camera_ray(Camera *cam, unsigned int *s0, unsigned int *s1, int w, int h,
                             int x, int y, Ray *ray) {
    rk0::GenerateCameraRay(cam, s0, s1, w, h, x, y, ray);
}

} /* extern "C" */
