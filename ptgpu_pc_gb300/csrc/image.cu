// image.cu -- the frame as an image file, encoded on the device.
//
// PPM: the reference's dump of the display buffer (smallptGPU.cpp:1238-1257):
// "P3\n<w> <h>\n255\n", then for every pixel, rows from the top of the image
// (y = h-1) down to y = 0, "<r> <g> <b> " in decimal, no line breaks.  The
// digits are written on the device: one CTA per output row counts its
// characters, one CTA turns the row counts into offsets, and one CTA per row
// scans its pixels' lengths and writes their text, so the file leaves the
// device in one copy.
// PFM: the running mean itself ("PF\n<w> <h>\n-1.0\n", float RGB,
// little-endian, bottom row first), gathered from the row-flipped colour
// buffer in one pass.
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "lbvh.h"

namespace ptgpu {

namespace {

constexpr int kRowThreads = 256;

__device__ __forceinline__ uint32_t dec_len(uint32_t v) { return v < 10u ? 1u : (v < 100u ? 2u : 3u); }

__device__ __forceinline__ uint32_t pixel_len(uint32_t p) {
    return dec_len(p & 255u) + dec_len((p >> 8) & 255u) + dec_len((p >> 16) & 255u) + 3u;
}

__device__ __forceinline__ char *put_dec(char *o, uint32_t v) {
    if (v >= 100u) { *o++ = (char)('0' + v / 100u); v %= 100u; *o++ = (char)('0' + v / 10u); v %= 10u; }
    else if (v >= 10u) { *o++ = (char)('0' + v / 10u); v %= 10u; }
    *o++ = (char)('0' + v);
    *o++ = ' ';
    return o;
}

// block-wide exclusive scan of one 64-bit value per thread; returns the
// block total through *total
__device__ uint64_t block_scan_excl(uint64_t v, uint64_t *total) {
    __shared__ uint64_t warp_sum[kRowThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[w] = x;
    __syncthreads();
    uint64_t base = 0, all = 0;
    for (int k = 0; k < kRowThreads / 32; ++k) {
        if (k < w) base += warp_sum[k];
        all += warp_sum[k];
    }
    __syncthreads();
    *total = all;
    return base + x - v;
}

// the pixels a thread of a row's CTA takes: a contiguous run
__device__ __forceinline__ void thread_run(int w, int &x0, int &x1) {
    const int per = (w + kRowThreads - 1) / kRowThreads;
    x0 = min(w, (int)threadIdx.x * per);
    x1 = min(w, x0 + per);
}

__global__ void __launch_bounds__(kRowThreads) k_ppm_row_len(const uint32_t *__restrict__ pixels, int w, int h,
                                                              uint64_t *__restrict__ row_len) {
    const int r = blockIdx.x;                  // output row r holds image row y = h-1-r
    const uint32_t *row = pixels + (size_t)(h - 1 - r) * w;
    int x0, x1;
    thread_run(w, x0, x1);
    uint64_t n = 0;
    for (int x = x0; x < x1; ++x) n += pixel_len(row[x]);
    uint64_t total;
    block_scan_excl(n, &total);
    if (threadIdx.x == 0) row_len[r] = total;
}

// row_len (h entries) -> exclusive offsets in place; the total to row_len[h]
__global__ void __launch_bounds__(kRowThreads) k_ppm_row_scan(uint64_t *row_len, int h) {
    uint64_t carry = 0;
    for (int base = 0; base < h; base += kRowThreads) {
        const int i = base + threadIdx.x;
        const uint64_t v = i < h ? row_len[i] : 0;
        uint64_t total;
        const uint64_t ex = block_scan_excl(v, &total);
        if (i < h) row_len[i] = carry + ex;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) row_len[h] = carry;
}

__global__ void __launch_bounds__(kRowThreads) k_ppm_write(const uint32_t *__restrict__ pixels, int w, int h,
                                                            const uint64_t *__restrict__ row_off,
                                                            char *__restrict__ out) {
    const int r = blockIdx.x;
    const uint32_t *row = pixels + (size_t)(h - 1 - r) * w;
    int x0, x1;
    thread_run(w, x0, x1);
    uint64_t n = 0;
    for (int x = x0; x < x1; ++x) n += pixel_len(row[x]);
    uint64_t total;
    char *o = out + row_off[r] + block_scan_excl(n, &total);
    for (int x = x0; x < x1; ++x) {
        const uint32_t p = row[x];
        o = put_dec(o, p & 255u);
        o = put_dec(o, (p >> 8) & 255u);
        o = put_dec(o, (p >> 16) & 255u);
    }
}

__global__ void k_pfm(const ptgpu_vec *__restrict__ colors, int w, int h, float *__restrict__ out) {
    const int64_t n = (int64_t)w * h;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int y = (int)(i / w), x = (int)(i % w);   // file order: bottom row (y = 0) first
        const ptgpu_vec c = colors[(int64_t)(h - 1 - y) * w + x];
        out[3 * i + 0] = c.x;
        out[3 * i + 1] = c.y;
        out[3 * i + 2] = c.z;
    }
}

}  // namespace

cudaError_t launch_ppm_length(const uint32_t *pixels, int w, int h, uint64_t *row_off, cudaStream_t s) {
    k_ppm_row_len<<<h, kRowThreads, 0, s>>>(pixels, w, h, row_off);
    k_ppm_row_scan<<<1, kRowThreads, 0, s>>>(row_off, h);
    return cudaGetLastError();
}

cudaError_t launch_ppm_write(const uint32_t *pixels, int w, int h, const uint64_t *row_off, char *out,
                             cudaStream_t s) {
    k_ppm_write<<<h, kRowThreads, 0, s>>>(pixels, w, h, row_off, out);
    return cudaGetLastError();
}

cudaError_t launch_pfm(const ptgpu_vec *colors, int w, int h, float *out, int sm_count, cudaStream_t s) {
    const int64_t n = (int64_t)w * h;
    int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count * 8);
    if (grid < 1) grid = 1;
    k_pfm<<<grid, 256, 0, s>>>(colors, w, h, out);
    return cudaGetLastError();
}

}  // namespace ptgpu
