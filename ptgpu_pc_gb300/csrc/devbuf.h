// devbuf.h -- a growable device buffer owned by a host object (contexts and
// batches): ensure() reallocates only when the buffer must grow.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

namespace ptgpu {

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t want) {
        if (want <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (want == 0) want = 16;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
};

}  // namespace ptgpu
