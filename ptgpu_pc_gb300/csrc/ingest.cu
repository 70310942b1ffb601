// ingest.cu -- scene ingestion without a host copy of the shape array.
//
// read_scene (displayfunc.cpp:144-505 ReadTxt, 717-730 Read) expands every OBJ
// model into full 104-byte Shape records on the host before they are copied to
// the device.  Here a scene arrives as segments (CompactScene): small runs of
// shapes read from the scene file, and models kept as the OBJ reader's vertex
// array (12 bytes per vertex) and triangle indices (12 bytes per triangle).
// Both are copied as they are; k_model_shapes expands each model triangle into
// its Shape record on the device with the host loader's arithmetic (scale,
// then translate; |cross(p2-p1, p3-p1)| * 0.5 with IEEE sqrt, no contraction),
// so the records are byte-identical to read_scene's.  Emitting model triangles
// get their light records (the SampleLights list, in index order) from
// k_model_lights; the few light records of plain shapes are made on the host.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "host.h"
#include "lbvh.h"
#include "ingest.h"

namespace ptgpu {

namespace {

struct ModelXf {
    float px, py, pz, sx, sy, sz;      // translate, scale
    float ex, ey, ez, cx, cy, cz;      // emission, colour
    int32_t refl;
};

__global__ void k_model_shapes(const float *__restrict__ v, const int32_t *__restrict__ tri, int64_t ntri,
                               int32_t nverts, ModelXf x, ptgpu_shape *__restrict__ out) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    float p[9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int32_t i = tri[3 * t + k];
        i = i < 0 ? 0 : (i >= nverts ? nverts - 1 : i);     // indices were checked on the host
        p[3 * k + 0] = v[3 * (size_t)i + 0] * x.sx + x.px;
        p[3 * k + 1] = v[3 * (size_t)i + 1] * x.sy + x.py;
        p[3 * k + 2] = v[3 * (size_t)i + 2] * x.sz + x.pz;
    }
    const float e1x = p[3] - p[0], e1y = p[4] - p[1], e1z = p[5] - p[2];
    const float e2x = p[6] - p[0], e2y = p[7] - p[1], e2z = p[8] - p[2];
    const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    const float area = sqrtf(nx * nx + ny * ny + nz * nz) * 0.5f;
    // the record as 26 words: type, p1..p3, e, c, refl, index 0, morton 0,
    // bound zeros, area
    uint32_t w[26];
    w[0] = PTGPU_TRIANGLE;
#pragma unroll
    for (int k = 0; k < 9; ++k) w[1 + k] = __float_as_uint(p[k]);
    w[10] = __float_as_uint(x.ex); w[11] = __float_as_uint(x.ey); w[12] = __float_as_uint(x.ez);
    w[13] = __float_as_uint(x.cx); w[14] = __float_as_uint(x.cy); w[15] = __float_as_uint(x.cz);
    w[16] = (uint32_t)x.refl;
#pragma unroll
    for (int k = 17; k < 25; ++k) w[k] = 0u;
    w[25] = __float_as_uint(area);
    uint32_t *dst = reinterpret_cast<uint32_t *>(out + t);
#pragma unroll
    for (int k = 0; k < 26; ++k) dst[k] = w[k];
}

// light records of `count` consecutive emitting triangles (make_lights' layout)
__global__ void k_model_lights(const ptgpu_shape *__restrict__ shapes, int64_t count, LightRec *__restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= count) return;
    const ptgpu_shape s = shapes[i];
    const ptgpu_triangle &t = s.g.t;
    LightRec L;
    L.a = make_float4(t.p1.x, t.p1.y, t.p1.z, __int_as_float(PTGPU_TRIANGLE));
    L.b = make_float4(t.p2.x - t.p1.x, t.p2.y - t.p1.y, t.p2.z - t.p1.z, s.area);
    L.c = make_float4(t.p3.x - t.p1.x, t.p3.y - t.p1.y, t.p3.z - t.p1.z, 0.f);
    L.e = make_float4(s.e.x, s.e.y, s.e.z, 0.f);
    out[i] = L;
}

bool emits(const ptgpu_vec &e) { return !(e.x == 0.f && e.y == 0.f && e.z == 0.f); }

}  // namespace

uint32_t compact_light_count(const CompactScene &sc) {
    uint64_t m = 0;
    for (const SceneSegment &g : sc.segs) {
        if (g.model) {
            if (emits(g.e)) m += (uint64_t)g.count();
        } else {
            for (const ptgpu_shape &s : g.shapes) m += emits(s.e) ? 1u : 0u;
        }
    }
    return (uint32_t)std::min<uint64_t>(m, sc.light_cnt);
}

bool compact_all_triangles(const CompactScene &sc) {
    for (const SceneSegment &g : sc.segs)
        if (!g.model)
            for (const ptgpu_shape &s : g.shapes)
                if (s.type != PTGPU_TRIANGLE) return false;
    return true;
}

cudaError_t ingest_compact(const CompactScene &sc, ptgpu_shape *d_shapes, LightRec *d_lights,
                           IngestScratch &scr, cudaStream_t s) {
    int64_t off = 0;
    uint32_t lights = 0;
    const uint32_t max_lights = compact_light_count(sc);
    std::vector<LightRec> host_lights;
    for (const SceneSegment &g : sc.segs) {
        const int64_t cnt = g.count();
        if (cnt == 0) continue;
        if (!g.model) {
            cudaError_t e = cudaMemcpyAsync(d_shapes + off, g.shapes.data(), (size_t)cnt * sizeof(ptgpu_shape),
                                            cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) return e;
            if (lights < max_lights) {
                make_lights(g.shapes.data(), (uint32_t)cnt, max_lights - lights, host_lights);
                if (!host_lights.empty()) {
                    // host_lights must outlive the copy: stage it in the scratch list
                    scr.host_lights.emplace_back(std::move(host_lights));
                    const std::vector<LightRec> &hl = scr.host_lights.back();
                    e = cudaMemcpyAsync(d_lights + lights, hl.data(), hl.size() * sizeof(LightRec),
                                        cudaMemcpyHostToDevice, s);
                    if (e != cudaSuccess) return e;
                    lights += (uint32_t)hl.size();
                    host_lights = std::vector<LightRec>();
                }
            }
        } else {
            const size_t vb = g.obj.v.size() * sizeof(float), tb = g.obj.tri.size() * sizeof(int32_t);
            // the scratch holds one model at a time: wait for the previous one
            cudaError_t e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return e;
            if ((e = scr.v.ensure(vb)) != cudaSuccess) return e;
            if ((e = scr.tri.ensure(tb)) != cudaSuccess) return e;
            if ((e = cudaMemcpyAsync(scr.v.p, g.obj.v.data(), vb, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
            if ((e = cudaMemcpyAsync(scr.tri.p, g.obj.tri.data(), tb, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
            ModelXf x;
            x.px = g.pos.x; x.py = g.pos.y; x.pz = g.pos.z;
            x.sx = g.scale.x; x.sy = g.scale.y; x.sz = g.scale.z;
            x.ex = g.e.x; x.ey = g.e.y; x.ez = g.e.z;
            x.cx = g.c.x; x.cy = g.c.y; x.cz = g.c.z;
            x.refl = g.refl;
            const int32_t nverts = (int32_t)(g.obj.v.size() / 3);
            k_model_shapes<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(scr.v.as<float>(), scr.tri.as<int32_t>(), cnt,
                                                                       nverts, x, d_shapes + off);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            if (emits(g.e) && lights < max_lights) {
                const int64_t m = std::min<int64_t>(cnt, (int64_t)(max_lights - lights));
                k_model_lights<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(d_shapes + off, m, d_lights + lights);
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
                lights += (uint32_t)m;
            }
        }
        off += cnt;
    }
    cudaError_t e = cudaStreamSynchronize(s);
    scr.host_lights.clear();
    return e;
}

}  // namespace ptgpu
