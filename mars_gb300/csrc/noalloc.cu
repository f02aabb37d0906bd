// Candidate projection that allocates no device memory.
//
// mars_gpu_orthonormalize_noalloc runs the same kernels as
// mars_gpu_orthonormalize (project, DGKS gate and retry, normalise) on device
// arrays the caller owns, on the caller's stream. Its working memory -- the
// FP64 projection coefficients T, the retried-column list and a few scalars --
// is one fixed array of module-scope device memory, so the call never reaches
// cudaMalloc or cudaFree.
#include "../../include/mars_gpu.h"
#include "common.cuh"
#include "fp64.cuh"

using namespace mgpu;

namespace {

// Limits of the fixed scratch (declared in mars_gpu.h as well).
constexpr size_t NA_MAX_CAND = MARS_GPU_NOALLOC_MAX_CANDIDATES;
constexpr size_t NA_MAX_T = MARS_GPU_NOALLOC_MAX_COEFS;

constexpr size_t na_align(size_t b) { return (b + 255) / 256 * 256; }

// Scratch layout, every region 256-byte aligned.
constexpr size_t OFF_T = 0;                                                // NA_MAX_T doubles
constexpr size_t OFF_SNEW = OFF_T + na_align(NA_MAX_T * sizeof(double));   // NA_MAX_CAND doubles
constexpr size_t OFF_S = OFF_SNEW + na_align(NA_MAX_CAND * sizeof(double));  // NA_MAX_CAND doubles
constexpr size_t OFF_CX = OFF_S + na_align(NA_MAX_CAND * sizeof(double));  // NA_MAX_CAND ints
constexpr size_t OFF_CB = OFF_CX + na_align(NA_MAX_CAND * sizeof(int));    // NA_MAX_CAND ints
constexpr size_t OFF_FIRED = OFF_CB + na_align(NA_MAX_CAND * sizeof(int));  // NA_MAX_CAND ints
constexpr size_t OFF_NF = OFF_FIRED + na_align(NA_MAX_CAND * sizeof(int));  // 1 int
constexpr size_t OFF_ONE = OFF_NF + 256;                                     // 1 float
constexpr size_t NA_BYTES = OFF_ONE + 256;

__device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

// Address of the scratch on the current device. Looked up on every call (a
// cheap runtime query), so a new primary context -- after cudaDeviceReset,
// say -- never leaves a stale address behind.
unsigned char *scratch_address()
{
    void *p = nullptr;
    CUDA_CHECK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    verify(p != nullptr, "scratch symbol has no device address", MARS_GPU_ECUDA);
    return static_cast<unsigned char *>(p);
}

const float kOne = 1.0f;

}  // namespace

extern "C" {

int mars_gpu_orthonormalize_noalloc(size_t n, size_t m, size_t p, const float *B, size_t ldB,
                                    size_t ncolB, const float *x, const int *mask, const float *Bo,
                                    size_t ldBo, float *Bx, size_t ldBx, double *s, double tol,
                                    void *stream, long *dgks)
{
    try {
        verify(mars_gpu_device_count() > 0, "no CUDA device is visible", MARS_GPU_ECUDA);
        verify(B && x && mask && Bx && (Bo || m == 0), "null argument");
        verify(n >= 1 && p >= 1, "empty problem");
        verify(n <= 0x7fffffff, "too many rows for one call");
        verify(ldB >= n && ldBx >= n && (m == 0 || ldBo >= m),
               "leading dimension smaller than the data");
        verify(p <= NA_MAX_CAND,
               "too many candidate columns for the fixed scratch (at most "
               "MARS_GPU_NOALLOC_MAX_CANDIDATES)");
        verify(m * p <= NA_MAX_T,
               "m * p exceeds the fixed scratch (at most MARS_GPU_NOALLOC_MAX_COEFS)");
        for (size_t j = 0; j < p; ++j) {
            verify(mask[j] >= 0 && (size_t)mask[j] < ncolB,
                   "basis index in mask outside the columns of B");
        }
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        unsigned char *base = scratch_address();
        double *T = reinterpret_cast<double *>(base + OFF_T);
        double *snew = reinterpret_cast<double *>(base + OFF_SNEW);
        double *sv = s ? s : reinterpret_cast<double *>(base + OFF_S);
        int *cand_x = reinterpret_cast<int *>(base + OFF_CX);
        int *cand_b = reinterpret_cast<int *>(base + OFF_CB);
        int *fired = reinterpret_cast<int *>(base + OFF_FIRED);
        int *nfired = reinterpret_cast<int *>(base + OFF_NF);
        float *one = reinterpret_cast<float *>(base + OFF_ONE);

        // Everything read from the scratch is written first by this call:
        // the candidate lists and the unit scale here, T by the projection,
        // the retry count by the DGKS gate (which clears it).
        CUDA_CHECK(cudaMemsetAsync(cand_x, 0, sizeof(int) * p, st));
        CUDA_CHECK(cudaMemcpyAsync(cand_b, mask, sizeof(int) * p, cudaMemcpyHostToDevice, st));
        CUDA_CHECK(cudaMemcpyAsync(one, &kOne, sizeof(float), cudaMemcpyHostToDevice, st));

        long long launches = 0;
        const size_t ldbo = m == 0 ? 1 : ldBo;
        ProjectScratch ws{T};
        FillSrc src{B, ldB, x, n, one, cand_x, cand_b};
        project_fp64(st, src, Bo, ldbo, nullptr, nullptr, (int)n, (int)m, (int)p, nullptr, Bx, ldBx,
                     sv, ws,
                     &launches);
        dgks_gate(st, T, (int)m, (int)p, sv, tol, fired, nfired, &launches);
        int nf = 0;
        CUDA_CHECK(cudaMemcpyAsync(&nf, nfired, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        if (nf > 0) {
            StoredSrc s2{Bx, ldBx, fired};
            project_fp64(st, s2, Bo, ldbo, nullptr, nullptr, (int)n, (int)m, nf, fired, Bx, ldBx,
                         snew, ws,
                         &launches);
            scatter_s(st, fired, nf, snew, sv, &launches);
        }
        scale_columns(st, Bx, ldBx, (int)n, (int)p, sv, tol, &launches);
        if (dgks) {
            *dgks += nf;
        }
        return MARS_GPU_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.status;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return MARS_GPU_ECUDA;
    }
}

}  // extern "C"
