/*
 * ref_cpu.cpp -- the reference's CPU path (include/geomfunc.h) driven like
 * DrawBox (smallptGPU.cpp:652-723): OpenMP over rows, one path per pixel per
 * pass.  Compiled three times (REF_ACCEL = 0, 1, 2) by oracle/ref/build_ref.sh.
 * TEST INFRASTRUCTURE ONLY: it is the timed CPU baseline when the reference
 * tree is available.
 */
#include <cmath>
#include "include/geom.h"
#include "include/camera.h"
#include "include/BVHNodeGPU.h"
#include "include/KDNodeGPU.h"
#undef ACCELSTR
#define ACCELSTR REF_ACCEL
#define REF_CAT2(a, b) a##b
#define REF_CAT(a, b) REF_CAT2(a, b)
#define REF_NS REF_CAT(gf, REF_ACCEL)
namespace REF_NS {
#include "include/geomfunc.h"
}

extern "C" void REF_CAT(ref_cpu_render_acc, REF_ACCEL)(
    const Camera *cam, Shape *shapes, unsigned int n, unsigned int light_cnt,
    BVHNodeGPU *btn, BVHNodeGPU *btl, KDNodeGPU *kng, int kng_cnt, int *kn, int kn_cnt,
    int w, int h, int row_begin, int row_end, int current_sample, Vec *colors,
    unsigned int *seeds, int threads) {
    (void)btn; (void)btl; (void)kng; (void)kng_cnt; (void)kn; (void)kn_cnt;
    const float invWidth = 1.f / w, invHeight = 1.f / h;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int y = row_begin; y < row_end; y++) {
        for (int x = 0; x < w; x++) {
            const int i = (h - y - 1) * w + x;
            const int i2 = i << 1;
            const float r1 = REF_NS::GetRandom(&seeds[i2], &seeds[i2 + 1]) - .5f;
            const float r2 = REF_NS::GetRandom(&seeds[i2], &seeds[i2 + 1]) - .5f;
            const float kcx = (x + r1) * invWidth - .5f;
            const float kcy = (y + r2) * invHeight - .5f;
            Vec rdir;
            vinit(rdir, cam->x.x * kcx + cam->y.x * kcy + cam->dir.x,
                  cam->x.y * kcx + cam->y.y * kcy + cam->dir.y,
                  cam->x.z * kcx + cam->y.z * kcy + cam->dir.z);
            Vec rorig;
            vsmul(rorig, 0.1f, rdir);
            vadd(rorig, rorig, cam->orig);
            vnorm(rdir);
            const Ray ray = {rorig, rdir};
            Vec r;
            r.x = r.y = r.z = 1.0f;
#if REF_ACCEL == 0
            REF_NS::RadiancePathTracing(shapes, n, light_cnt, &ray, &seeds[i2], &seeds[i2 + 1], &r);
#elif REF_ACCEL == 1
            REF_NS::RadiancePathTracing(shapes, n, light_cnt, btn, btl, &ray, &seeds[i2],
                                        &seeds[i2 + 1], &r);
#else
            REF_NS::RadiancePathTracing(shapes, n, light_cnt, kng, kn, kng_cnt, kn_cnt, &ray,
                                        &seeds[i2], &seeds[i2 + 1], &r);
#endif
            if (current_sample == 0) colors[i] = r;
            else {
                const float k1 = current_sample;
                const float k2 = 1.f / (k1 + 1.f);
                colors[i].x = (colors[i].x * k1 + r.x) * k2;
                colors[i].y = (colors[i].y * k1 + r.y) * k2;
                colors[i].z = (colors[i].z * k1 + r.z) * k2;
            }
        }
    }
}
