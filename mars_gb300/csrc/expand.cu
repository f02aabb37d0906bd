// Differentiable basis expansion of a fitted model (mars.py:423-450 expand,
// with the prediction B beta) and its backward pass.
//
// A model is M terms in order; term j has a kind (intercept, linear, '+'
// hinge, '-' hinge), a parent term p_j < j, an input column c_j and a knot t_j:
//   B_0 = 1,   B_j = B_{p_j} * f_j(x_{c_j}),
//   f = x (linear), max(x - t, 0) ('+'), max(t - x, 0) ('-'),
//   pred = sum_j beta_j B_j.
// Backward, per row, with the adjoint a_j = d pred / d B_j taken in reverse
// term order (a_j = beta_j + sum over children k of a_k f_k):
//   d pred / d beta_j = B_j
//   d pred / d t_k    = a_k B_{p_k} df_k/dt   (-1{x > t} for '+', +1{x < t} for '-')
//   d pred / d x_c    = sum over terms k on input c of a_k B_{p_k} df_k/dx
// scaled by the incoming gradient of each row. The beta and knot gradients are
// summed over rows per block and then across blocks in a fixed order.
#include "../../include/mars_gpu.h"
#include "common.cuh"

#include <algorithm>

namespace mgpu {
namespace {

constexpr int EX_THREADS = 256, EX_MAXM = 128;

struct Terms {
    const int *kind;    // MARS_GPU_TERM_*
    const int *parent;  // parent term index (< own index)
    const int *input;   // X column
    const float *knot;  // hinge knot (ignored otherwise)
    const float *beta;  // coefficients
    int M;
};

__device__ __forceinline__ float term_factor(int kind, float x, float t)
{
    switch (kind) {
    case MARS_GPU_TERM_LINEAR:
        return x;
    case MARS_GPU_TERM_PLUS:
        return fmaxf(x - t, 0.0f);
    case MARS_GPU_TERM_MINUS:
        return fmaxf(t - x, 0.0f);
    default:
        return 1.0f;
    }
}

// df/dx and df/dt of a term factor (subgradient 0 at the knot).
__device__ __forceinline__ void term_slopes(int kind, float x, float t, float *dx, float *dt)
{
    *dx = 0.f;
    *dt = 0.f;
    if (kind == MARS_GPU_TERM_LINEAR) {
        *dx = 1.f;
    } else if (kind == MARS_GPU_TERM_PLUS && x > t) {
        *dx = 1.f;
        *dt = -1.f;
    } else if (kind == MARS_GPU_TERM_MINUS && x < t) {
        *dx = -1.f;
        *dt = 1.f;
    }
}

__global__ void __launch_bounds__(EX_THREADS)
    k_expand(Terms tm, const float *__restrict__ X, size_t ldx, size_t N, float *__restrict__ pred,
             float *__restrict__ B, size_t ldb)
{
    float b[EX_MAXM];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (size_t)gridDim.x * blockDim.x) {
        float p = 0.f;
        for (int j = 0; j < tm.M; ++j) {
            const int k = tm.kind[j];
            const float v = k == MARS_GPU_TERM_INTERCEPT
                                ? 1.0f
                                : b[tm.parent[j]] *
                                      term_factor(k, X[i + (size_t)tm.input[j] * ldx], tm.knot[j]);
            b[j] = v;
            p = fmaf(tm.beta[j], v, p);
            if (B) {
                B[i + (size_t)j * ldb] = v;
            }
        }
        if (pred) {
            pred[i] = p;
        }
    }
}

__global__ void __launch_bounds__(EX_THREADS)
    k_expand_backward(Terms tm, const float *__restrict__ X, size_t ldx, size_t N,
                      const float *__restrict__ g, float *__restrict__ dX, size_t lddx,
                      double *__restrict__ part)
{
    __shared__ double red[EX_THREADS / 32];
    float b[EX_MAXM], a[EX_MAXM];
    double gb[EX_MAXM], gt[EX_MAXM];  // this thread's sums over its rows
    for (int j = 0; j < tm.M; ++j) {
        gb[j] = 0.0;
        gt[j] = 0.0;
    }
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < N;
         i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        for (int j = 0; j < tm.M; ++j) {
            const int k = tm.kind[j];
            b[j] = k == MARS_GPU_TERM_INTERCEPT
                       ? 1.0f
                       : b[tm.parent[j]] *
                             term_factor(k, X[i + (size_t)tm.input[j] * ldx], tm.knot[j]);
            a[j] = tm.beta[j];
        }
        for (int j = tm.M - 1; j >= 1; --j) {
            const int k = tm.kind[j];
            if (k != MARS_GPU_TERM_INTERCEPT) {
                const float x = X[i + (size_t)tm.input[j] * ldx];
                a[tm.parent[j]] = fmaf(a[j], term_factor(k, x, tm.knot[j]), a[tm.parent[j]]);
            }
        }
        for (int j = 0; j < tm.M; ++j) {
            gb[j] += (double)gi * (double)b[j];
            const int k = tm.kind[j];
            if (k == MARS_GPU_TERM_INTERCEPT) {
                continue;
            }
            const int c = tm.input[j];
            const float x = X[i + (size_t)c * ldx];
            float sx, st;
            term_slopes(k, x, tm.knot[j], &sx, &st);
            const float w = gi * a[j] * b[tm.parent[j]];
            gt[j] += (double)(w * st);
            if (dX && sx != 0.f) {
                dX[i + (size_t)c * lddx] += w * sx;
            }
        }
    }
    // per-block sums, fixed order
    for (int j = 0; j < 2 * tm.M; ++j) {
        double v = j < tm.M ? gb[j] : gt[j - tm.M];
        v = warp_sum(v);
        if ((threadIdx.x & 31) == 0) {
            red[threadIdx.x >> 5] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < EX_THREADS / 32; ++w) {
                s += red[w];
            }
            part[(size_t)blockIdx.x * 2 * tm.M + j] = s;
        }
        __syncthreads();
    }
}

__global__ void k_expand_reduce(const double *__restrict__ part, int nblocks, int M,
                                double *__restrict__ dbeta, double *__restrict__ dknot)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 2 * M) {
        return;
    }
    double s = 0.0;
    for (int q = 0; q < nblocks; ++q) {
        s += part[(size_t)q * 2 * M + j];
    }
    if (j < M) {
        dbeta[j] = s;
    } else {
        dknot[j - M] = s;
    }
}

int expand_blocks(size_t N)
{
    return (int)std::max<size_t>(1, std::min<size_t>(4 * 152, ceil_div(N, EX_THREADS)));
}

void check_terms(int M)
{
    verify(M >= 1 && M <= EX_MAXM, "the expansion supports 1 to 128 terms");
}

template <class F>
int guarded_call(F &&f)
{
    try {
        f();
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

using namespace mgpu;

extern "C" {

size_t mars_gpu_expand_workspace(size_t N, int M)
{
    return sizeof(double) * 2 * (size_t)std::max(M, 1) * expand_blocks(N);
}

int mars_gpu_expand(const int *kind, const int *parent, const int *input, const float *knot,
                    const float *beta, int M, const float *X, size_t ldx, size_t N, float *pred,
                    float *B, size_t ldb, void *stream)
{
    return guarded_call([&] {
        check_terms(M);
        verify(X && kind && parent && input && knot && beta, "null argument");
        verify(ldx >= N && (!B || ldb >= N), "leading dimension smaller than the data");
        if (N == 0) {
            return;
        }
        Terms tm{kind, parent, input, knot, beta, M};
        k_expand<<<expand_blocks(N), EX_THREADS, 0, static_cast<cudaStream_t>(stream)>>>(
            tm, X, ldx, N, pred, B, ldb);
        LAUNCH_CHECK();
    });
}

int mars_gpu_expand_backward(const int *kind, const int *parent, const int *input,
                             const float *knot, const float *beta, int M, const float *X,
                             size_t ldx, size_t N, const float *g, float *dX, size_t lddx,
                             double *dbeta, double *dknot, void *workspace, void *stream)
{
    return guarded_call([&] {
        check_terms(M);
        verify(X && kind && parent && input && knot && beta && g && dbeta && dknot && workspace,
               "null argument");
        verify(ldx >= N && (!dX || lddx >= N), "leading dimension smaller than the data");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const int nb = expand_blocks(std::max<size_t>(N, 1));
        Terms tm{kind, parent, input, knot, beta, M};
        double *part = static_cast<double *>(workspace);
        if (N > 0) {
            k_expand_backward<<<nb, EX_THREADS, 0, st>>>(tm, X, ldx, N, g, dX, lddx, part);
            LAUNCH_CHECK();
        } else {
            CUDA_CHECK(cudaMemsetAsync(part, 0, sizeof(double) * 2 * M * nb, st));
        }
        k_expand_reduce<<<(unsigned)ceil_div(2 * M, 128), 128, 0, st>>>(part, N > 0 ? nb : 1, M,
                                                                       dbeta, dknot);
        LAUNCH_CHECK();
    });
}

}  // extern "C"
