// Gram matrix of the backward pass: G = A^T B in the reference's arithmetic.
//
// The reference's gram (mars.py:456-490) multiplies 128-row chunks in the
// input dtype (numpy's BLAS) and adds each chunk's product, widened to
// float64, to a float64 total in chunk order. Each entry of a chunk product
// is, in that BLAS, one fused multiply-add chain over the chunk's rows in
// order (verified bit for bit against numpy's float32 and float64 products on
// the golden bases). The backward elimination that follows is ill-conditioned
// on hinge pairs near the sorted ends -- a Gram matrix rounded differently by
// 1e-8 flips a pruning decision of the hinge-search golden fit -- so this
// kernel reproduces that arithmetic: per entry, per 128-row chunk, an FMA
// chain in the input dtype, then the FP64 chunk-order total. One thread per
// entry, the chunk's rows staged in shared memory. The reference forms its
// matrix-vector and vector-vector products (X^T y, y^T y) with other BLAS
// kernels that keep several partial sums; those run here with `exact` set:
// products widened exactly, FP64 chains (closer to any such order than an
// f32 chain is).
#include "../../include/mars_gpu.h"
#include "common.cuh"

#include <algorithm>

namespace mgpu {
namespace {

constexpr int GR_T = 16;       // output tile: 16 x 16 entries, one per thread
constexpr int GR_CHUNK = 128;  // the reference's chunk of rows

__device__ __forceinline__ float fma_e(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_e(double a, double b, double c) { return __fma_rn(a, b, c); }

// Acc = E: the reference's chunk chains; Acc = double: every product widened
// exactly and the chunk chain in FP64 (the matrix-vector products, whose
// reference BLAS order is not a plain chain).
template <class E, class Acc>
__global__ void __launch_bounds__(GR_T *GR_T)
    k_gram(const E *__restrict__ A, size_t lda, int ka, const E *__restrict__ B, size_t ldb,
           int kb, int n, double *__restrict__ out)
{
    __shared__ E sA[GR_CHUNK][GR_T + 1];
    __shared__ E sB[GR_CHUNK][GR_T + 1];
    const int tx = threadIdx.x % GR_T, ty = threadIdx.x / GR_T;
    const int i0 = blockIdx.x * GR_T, j0 = blockIdx.y * GR_T;
    double total = 0.0;
    for (int c0 = 0; c0 < n; c0 += GR_CHUNK) {
        const int rows = min(GR_CHUNK, n - c0);
        for (int e = threadIdx.x; e < GR_CHUNK * GR_T; e += GR_T * GR_T) {
            const int rr = e % GR_CHUNK, c = e / GR_CHUNK, r = c0 + rr;
            sA[rr][c] = (rr < rows && i0 + c < ka) ? A[(size_t)(i0 + c) * lda + r] : E(0);
            sB[rr][c] = (rr < rows && j0 + c < kb) ? B[(size_t)(j0 + c) * ldb + r] : E(0);
        }
        __syncthreads();
        Acc acc = Acc(0);
        for (int rr = 0; rr < rows; ++rr) {
            acc = fma_e((Acc)sA[rr][ty], (Acc)sB[rr][tx], acc);
        }
        total = __dadd_rn(total, (double)acc);
        __syncthreads();
    }
    const int i = i0 + ty, j = j0 + tx;
    if (i < ka && j < kb) {
        out[(size_t)i * kb + j] = total;
    }
}

template <class E>
int gram_impl(size_t n, const E *A, size_t lda, size_t ka, const E *B, size_t ldb, size_t kb,
              int exact, double *out)
{
    try {
        verify(mars_gpu_device_count() > 0, "no CUDA device is visible", MARS_GPU_ECUDA);
        verify(A && B && out, "null argument");
        verify(lda >= n && ldb >= n, "leading dimension smaller than the data");
        verify(n <= 0x7fffffff && ka <= 65535 * (size_t)GR_T && kb <= 65535 * (size_t)GR_T,
               "gram: too many rows or columns");
        if (ka == 0 || kb == 0) {
            return MARS_GPU_OK;
        }
        cudaStream_t st = nullptr;
        CUDA_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
        } guard{st};
        DevBuf dA, dB, dOut;
        for (DevBuf *b : {&dA, &dB, &dOut}) {
            b->bind(st);
        }
        const size_t nn = std::max<size_t>(n, 1), es = sizeof(E);
        dA.ensure(es * nn * ka);
        dB.ensure(es * nn * kb);
        if (n) {
            CUDA_CHECK(cudaMemcpy2DAsync(dA.ptr, n * es, A, lda * es, n * es, ka,
                                         cudaMemcpyHostToDevice, st));
            CUDA_CHECK(cudaMemcpy2DAsync(dB.ptr, n * es, B, ldb * es, n * es, kb,
                                         cudaMemcpyHostToDevice, st));
        }
        const size_t cnt = ka * kb;
        dOut.ensure(sizeof(double) * cnt);
        const dim3 grid((unsigned)ceil_div(ka, GR_T), (unsigned)ceil_div(kb, GR_T));
        if (exact) {
            k_gram<E, double><<<grid, GR_T * GR_T, 0, st>>>(dA.as<E>(), n, (int)ka, dB.as<E>(),
                                                            n, (int)kb, (int)n,
                                                            dOut.as<double>());
        } else {
            k_gram<E, E><<<grid, GR_T * GR_T, 0, st>>>(dA.as<E>(), n, (int)ka, dB.as<E>(), n,
                                                       (int)kb, (int)n, dOut.as<double>());
        }
        LAUNCH_CHECK();
        CUDA_CHECK(cudaMemcpyAsync(out, dOut.ptr, sizeof(double) * cnt, cudaMemcpyDeviceToHost,
                                   st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        return MARS_GPU_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.status;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return MARS_GPU_ECUDA;
    }
}

}  // namespace
}  // namespace mgpu

extern "C" {

MARS_GPU_API int mars_gpu_gram(size_t n, const float *A, size_t lda, size_t ka, const float *B,
                               size_t ldb, size_t kb, int exact, double *out)
{
    return mgpu::gram_impl(n, A, lda, ka, B, ldb, kb, exact, out);
}

MARS_GPU_API int mars_gpu_gram_f64(size_t n, const double *A, size_t lda, size_t ka,
                                   const double *B, size_t ldb, size_t kb, int exact,
                                   double *out)
{
    return mgpu::gram_impl(n, A, lda, ka, B, ldb, kb, exact, out);
}

}  // extern "C"
