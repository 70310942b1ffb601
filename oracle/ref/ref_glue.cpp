/*
 * ref_glue.cpp -- C ABI over the reference's host code (CLBVH.cpp, KDTree.cpp,
 * displayfunc.cpp), compiled unmodified from the reference tree by
 * oracle/ref/build_ref.sh.  TEST INFRASTRUCTURE ONLY.
 */
#include "stdafx.h"
#include "include\\CLBVH.h"
#include "include\\KDTree.h"
#include "include/camera.h"
#include "include/displayfunc.h"
#include <cstring>
#include <cstdlib>

/* globals the reference's translation units expect (smallptGPU.cpp:116-119) */
Camera camera;
Shape *shapes = nullptr;
unsigned int shapeCnt = 0, lightCnt = 0;
unsigned int renderingFlags = 0;

/* ReadPly (plyfile.c, third-party) is out of scope: stubs that fail cleanly. */
#include "include\\ply.h"
PlyFile *ply_open_for_reading(char *, int *, char ***, int *, float *) { return nullptr; }
PlyProperty **ply_get_element_description(PlyFile *, char *, int *, int *) { return nullptr; }
void ply_get_property(PlyFile *, char *, PlyProperty *) {}
void ply_get_element(PlyFile *, void *) {}
void ply_close(PlyFile *) {}
int equal_strings(char *, char *) { return 0; }

extern "C" cl_kernel ref_make_kernel(int which);
extern "C" void ref_free_kernel(cl_kernel k);

extern "C" {

/* CLBVH pipeline: constructor (bounds + Morton), radix tree, optionally the
 * bubble sort + refit kernel, getTrees. */
int ref_clbvh(Shape *sh, int n, BVHNodeGPU *btn, BVHNodeGPU *btl, int do_refit) {
    cl_kernel kr = ref_make_kernel(0), kb = ref_make_kernel(1), ko = ref_make_kernel(2);
    CLBVH *cb = new CLBVH(sh, n, nullptr, nullptr, kr, kb, ko);
    cb->buildRadixTree();
    if (do_refit) cb->buildBVHTree();
    BVHNodeGPU *pn = nullptr, *pl = nullptr;
    cb->getTrees(&pn, &pl);
    if (n > 1) std::memcpy(btn, pn, sizeof(BVHNodeGPU) * (n - 1));
    std::memcpy(btl, pl, sizeof(BVHNodeGPU) * n);
    delete cb;
    ref_free_kernel(kr); ref_free_kernel(kb); ref_free_kernel(ko);
    return 0;
}

/* CLBVH::bubblesort_Geometry on the shapes' Morton codes */
int ref_bubblesort(Shape *sh, int n, int *sorted) {
    cl_kernel kr = ref_make_kernel(0), kb = ref_make_kernel(1), ko = ref_make_kernel(2);
    CLBVH *cb = new CLBVH(sh, n, nullptr, nullptr, kr, kb, ko);
    Geometry *geo = new Geometry[n];
    for (int i = 0; i < n; i++) { geo[i].key_mc = sh[i].morton_code; geo[i].value = i; }
    int *s = cb->bubblesort_Geometry(geo);
    std::memcpy(sorted, s, sizeof(int) * n);
    delete[] s; delete[] geo; delete cb;
    ref_free_kernel(kr); ref_free_kernel(kb); ref_free_kernel(ko);
    return 0;
}

/* BuildKDtree (smallptGPU.cpp:1477-1493).  Returns malloc'd arrays. */
int ref_kd_build(Shape *sh, int n, KDNodeGPU **kng, int *kng_cnt, int **kn, int *kn_cnt) {
    std::vector<Shape *> vs;
    for (int i = 0; i < n; i++) { sh[i].index = i; sh[i].morton_code = 0; vs.push_back(&sh[i]); }
    KDTree *kd = new KDTree();
    KDTreeNode *root = kd->build(vs, 0);
    kd->getTrees(root, kng, kng_cnt, kn, kn_cnt);
    return 0;
}

void ref_free(void *p) { std::free(p); }

/* Read (displayfunc.cpp:717-730) with the render size preset like main(). */
int ref_read_scene(const char *path, int w, int h, Shape **out, unsigned int *n,
                   unsigned int *light, Camera *cam, int *walllight) {
    width = w; height = h;
    shapes = nullptr; shapeCnt = 0; lightCnt = 0;
    std::memset(&camera, 0, sizeof(camera));
    bool wl = true;
    char buf[1024];
    std::strncpy(buf, path, sizeof(buf) - 1); buf[sizeof(buf) - 1] = 0;
    bool ok = Read(buf, &wl);
    *out = shapes; *n = shapeCnt; *light = lightCnt; *cam = camera; *walllight = wl ? 1 : 0;
    return ok ? 0 : -1;
}

void ref_update_camera(Camera *cam) { camera = *cam; UpdateCamera(); *cam = camera; }

} /* extern "C" */
