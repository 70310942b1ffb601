// noalloc.cu -- an LBVH build that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc: an engine that owns every
// byte of device memory through its own pool or fixed budget and hands the
// library only buffers it has already placed; a real-time frame loop that must
// not stall on the device-wide synchronisation cudaMalloc/cudaFree can cause;
// a plug-in host that forbids its plug-ins to allocate.  For them
// ptgpu_build_bvh_noalloc builds the reference BVH (CLBVH.cpp: Morton codes,
// radix sort, radix tree, refit) from shapes and into node arrays that the
// caller has put in device memory.  Every intermediate -- vertices, bounds,
// Morton keys, sort buffers, look-back words, block bounds -- lives in one
// file-scope __device__ array of fixed size, carved per call below.
//
// The array exists once per device the library is loaded on and is held until
// the process exits.  Every call shares it and it keeps the last call's
// contents; the build itself clears what must start at zero (the state word
// block, the look-back words, the arrival counters) before using them.
// Calls that overlap on the GPU -- on two streams, or on one stream from two
// host threads without ordering -- race on the array: serialise them.
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "lbvh.h"

namespace ptgpu {

namespace {

// 31.8 MiB are needed at kNoAllocMaxShapes; the rest is slack
constexpr uint32_t kNoAllocMaxShapes = 1u << 18;
constexpr size_t kNoAllocScratchBytes = size_t(33) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// device address of the array, per device
std::mutex g_mutex;
void *g_scratch_addr[64] = {nullptr};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// The carve for n shapes; returns the bytes used.
size_t carve(unsigned char *base, size_t n, LbvhBuffers &b) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + off;
        off += align256(bytes);
        return p;
    };
    b.verts = reinterpret_cast<float *>(take(n * 9 * sizeof(float)));
    b.type = take(n);
    b.aabbs = reinterpret_cast<float4 *>(take(n * 2 * sizeof(float4)));
    b.leaf_bounds = reinterpret_cast<float4 *>(take(n * 2 * sizeof(float4)));
    b.keys = reinterpret_cast<uint32_t *>(take(n * 4));
    b.keys_alt = reinterpret_cast<uint32_t *>(take(n * 4));
    b.keys_tmp = reinterpret_cast<uint32_t *>(take(n * 4));
    b.vals_alt = reinterpret_cast<int32_t *>(take(n * 4));
    b.vals_tmp = reinterpret_cast<int32_t *>(take(n * 4));
    b.sorted = reinterpret_cast<int32_t *>(take(n * 4));
    b.status = reinterpret_cast<uint32_t *>(take(sort_status_words((int)n) * 4));
    b.state = reinterpret_cast<BuildState *>(take(sizeof(BuildState)));
    b.block_bounds = reinterpret_cast<float *>(take(block_bound_count((int)n) * 6 * sizeof(float)));
    b.arrivals = reinterpret_cast<uint32_t *>(take(block_bound_count((int)n) * sizeof(uint32_t)));
    return off;
}

// AoS shapes -> the build's vertex and type arrays (the k_unpack_shapes
// layout without the tracer's primitive and material records)
__global__ void k_noalloc_unpack(const ptgpu_shape *__restrict__ shapes, int n,
                                 float *__restrict__ verts, uint8_t *__restrict__ type) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ptgpu_shape s = shapes[i];
    float *v = verts + 9 * (size_t)i;
    type[i] = (uint8_t)s.type;
    if (s.type == PTGPU_TRIANGLE) {
        const ptgpu_triangle &t = s.g.t;
        v[0] = t.p1.x; v[1] = t.p1.y; v[2] = t.p1.z;
        v[3] = t.p2.x; v[4] = t.p2.y; v[5] = t.p2.z;
        v[6] = t.p3.x; v[7] = t.p3.y; v[8] = t.p3.z;
    } else {
        const ptgpu_sphere &sp = s.g.s;
        v[0] = sp.p.x; v[1] = sp.p.y; v[2] = sp.p.z; v[3] = sp.rad;
        v[4] = v[5] = v[6] = v[7] = v[8] = 0.f;
    }
}

int dev_fail(cudaError_t e, const char *what) {
    return record_error(PTGPU_E_DEVICE, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace
}  // namespace ptgpu

using namespace ptgpu;

extern "C" int ptgpu_build_bvh_noalloc(const ptgpu_shape *d_shapes, uint32_t n,
                                       ptgpu_bvh_node *d_btn, ptgpu_bvh_node *d_btl,
                                       void *stream) {
    if (n == 0) return record_error(PTGPU_E_INVAL, "ptgpu_build_bvh_noalloc: zero shapes");
    if (!d_shapes || !d_btn || !d_btl)
        return record_error(PTGPU_E_INVAL, "ptgpu_build_bvh_noalloc: null device buffer");
    if (n > kNoAllocMaxShapes)
        return record_error(PTGPU_E_RANGE, "ptgpu_build_bvh_noalloc: " + std::to_string(n) +
                                               " shapes exceed the fixed scratch limit of " +
                                               std::to_string(kNoAllocMaxShapes));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return dev_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return record_error(PTGPU_E_DEVICE, "device ordinal beyond 63");
    unsigned char *base = nullptr;
    {
        // Set-up, on the first call for this device (which is current here):
        // the address of the array as this device sees it.  The lookup may
        // initialise the module on the device, so a caller that captures
        // streams makes its first call before any capture begins.
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return dev_fail(e, "cudaGetSymbolAddress(scratch)");
            g_scratch_addr[dev] = p;
        }
        base = static_cast<unsigned char *>(g_scratch_addr[dev]);
    }
    LbvhBuffers b;
    if (carve(base, n, b) > kNoAllocScratchBytes)
        return record_error(PTGPU_E_RANGE, "ptgpu_build_bvh_noalloc: scratch layout exceeds the array");
    b.btn = d_btn;
    b.btl = d_btl;
    int sms = 1;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return dev_fail(e, "cudaDeviceGetAttribute");
    k_noalloc_unpack<<<(n + 255) / 256, 256, 0, s>>>(d_shapes, (int)n, const_cast<float *>(b.verts),
                                                     const_cast<uint8_t *>(b.type));
    e = cudaGetLastError();
    if (e != cudaSuccess) return dev_fail(e, "k_noalloc_unpack");
    e = launch_lbvh_build(b, (int)n, 0, sms, s);
    if (e != cudaSuccess) return dev_fail(e, "launch_lbvh_build");
    // the sort's error word (bit 0: a look-back wait gave up), read into the
    // host stack; this also makes the call return with the build finished
    uint32_t err_word = 0;
    e = cudaMemcpyAsync(&err_word, &b.state->error, sizeof(err_word), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return dev_fail(e, "reading the build state");
    if (err_word) return record_error(PTGPU_E_TIMEOUT, "radix sort look-back wait gave up");
    return PTGPU_OK;
}
