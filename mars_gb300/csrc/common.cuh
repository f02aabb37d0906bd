// Shared helpers for the GB300 MARS forward-pass kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <map>
#include <mutex>
#include <utility>
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

// Raises a kernel's dynamic shared-memory limit to at least `bytes`. The
// attribute is per kernel and process-wide, so concurrent handles launching
// the same kernel with different sizes would race if each set its own size;
// here it only ever grows (under a lock), to the largest size asked so far.
// Not to the device maximum: a larger limit can make the driver pick a larger
// shared-memory carveout and leave the kernel less L1 cache.
template <class K>
void allow_smem(K kernel, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> set;  // (device, kernel) -> bytes
    int dev = 0;
    CUDA_CHECK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = set[{dev, reinterpret_cast<const void *>(kernel)}];
    if (bytes > cur) {
        CUDA_CHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)bytes));
        cur = bytes;
    }
}

inline size_t ceil_div(size_t a, size_t b) { return (a + b - 1) / b; }
inline size_t round_up(size_t a, size_t b) { return ceil_div(a, b) * b; }

// The library's memory pool on the current device: stream-ordered
// allocations, so that a fit's buffers come and go without the device-wide
// synchronisation of cudaMalloc / cudaFree (which would stall every other
// fit running concurrently). Up to 8 GB of freed memory stays cached in it.
inline cudaMemPool_t device_pool()
{
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    int dev = 0;
    CUDA_CHECK(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    auto it = pools.find(dev);
    if (it != pools.end()) {
        return it->second;
    }
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    CUDA_CHECK(cudaMemPoolCreate(&pool, &props));
    unsigned long long keep = 8ull << 30;
    CUDA_CHECK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    pools[dev] = pool;
    return pool;
}

// Grow-only device buffer. Bound to a stream (bind), it is allocated from
// the library's pool and freed in that stream's order; unbound, with
// cudaMalloc / cudaFree.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    cudaStream_t st = nullptr;
    bool bound = false;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void bind(cudaStream_t s)
    {
        st = s;
        bound = true;
    }
    void release()
    {
        if (ptr) {
            if (bound) {
                cudaFreeAsync(ptr, st);
            } else {
                cudaFree(ptr);
            }
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
        cudaError_t e = bound ? cudaMallocFromPoolAsync(&ptr, want, device_pool(), st)
                              : cudaMalloc(&ptr, want);
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
// Asynchronous global -> shared copies (cp.async, sm_80+). A copy with
// `valid` false writes zero and reads nothing.
// ---------------------------------------------------------------------------
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem, bool valid = true)
{
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async size");
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int bytes = valid ? BYTES : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s), "l"(gmem), "n"(BYTES),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem, bool valid = true)
{
    cp_async<4>(smem, gmem, valid);
}
__device__ __forceinline__ void cp_async_commit()
{
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// Wait until at most N of this thread's committed groups are pending.
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ---------------------------------------------------------------------------
// Deterministic warp reduction (fixed butterfly order).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    return v;
}

}  // namespace mgpu
