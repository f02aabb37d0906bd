// Shared helpers for the GB300 MARS forward-pass kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "error.h"

namespace mgpu {

inline void cuda_check(cudaError_t e, const char *what, const char *file, int line)
{
    if (e != cudaSuccess) {
        int st = (e == cudaErrorMemoryAllocation) ? 3 : 2;
        throw Error(st, std::string(what) + ": " + cudaGetErrorString(e) + " (" + file + ":" +
                            std::to_string(line) + ")");
    }
}
#define CUDA_CHECK(x) ::mgpu::cuda_check((x), #x, __FILE__, __LINE__)
#define LAUNCH_CHECK() ::mgpu::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__)

inline size_t ceil_div(size_t a, size_t b) { return (a + b - 1) / b; }
inline size_t round_up(size_t a, size_t b) { return ceil_div(a, b) * b; }

// Grow-only device buffer.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (ptr) {
            cudaFree(ptr);
        }
        ptr = nullptr;
        bytes = 0;
    }
    void ensure(size_t want)
    {
        if (want <= bytes) {
            return;
        }
        release();
        if (want == 0) {
            return;
        }
        cudaError_t e = cudaMalloc(&ptr, want);
        if (e != cudaSuccess) {
            cudaGetLastError();  // clear the sticky-free allocation error
            ptr = nullptr;
            throw Error(3, "device allocation of " + std::to_string(want) + " bytes failed: " +
                               cudaGetErrorString(e));
        }
        bytes = want;
    }
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

// ---------------------------------------------------------------------------
// Deterministic block reductions (fixed tree order for a fixed block size).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    return v;
}

// Sum over the block; the result is valid in thread 0. `red` holds >= 32 doubles.
template <int BLOCK>
__device__ __forceinline__ double block_sum(double v, double *red)
{
    static_assert(BLOCK % 32 == 0 && BLOCK <= 1024, "block size");
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    if (lane == 0) {
        red[wid] = v;
    }
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = lane < BLOCK / 32 ? red[lane] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

}  // namespace mgpu
