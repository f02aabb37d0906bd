// Tensor-core (tcgen05) projection of the mixed-precision fast pass.
//
// The fast pass projects every candidate column v_j onto the complement of
// the orthonormal basis Bo (kernels.cc:283-417 restated in FP32 terms):
//   T  = Bo^T v            (m x P, a dense contraction over the n rows)
//   Bx = v - Bo T          (n x P)
// applied twice, the second pass on the first one's residual (the role of the
// reference's DGKS retry). On sm_103a both contractions run on the 5th
// generation tensor cores: tcgen05.mma, kind::tf32, with the FP32 values
// split into two TF32 terms (hi = the value with its low 13 mantissa bits
// cleared, lo = value - hi, exact in FP32) and the three products
// hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory: about 22
// mantissa bits per product, the accuracy of the FP32 SIMT kernels these
// replace. The Bo operands are TMA-fed (cp.async.bulk.tensor) from split
// copies of the basis kept next to the fit state; the candidate operand is
// formed from its source columns by the producer warps.
#pragma once

#include "common.cuh"
#include "fast.cuh"
#include "fp64.cuh"

namespace mgpu {

// Split copies of the orthonormal basis, updated column by column at append.
struct TcBasis {
    float *hiC = nullptr, *loC = nullptr;  // column-major, leading dimension ldn (rows, >= n)
    float *hiR = nullptr, *loR = nullptr;  // row-major, leading dimension ldk (columns)
    size_t ldn = 0, ldk = 0;
};

// Scratch of one tensor-core projection of P candidates.
struct TcScratch {
    float *Tp;   // split-K partials [ks][P][m]
    float *T;    // [P][m] (f32 coefficients of the last pass)
    float *Thi;  // [P][ldk] split of T, zero past m
    float *Tlo;
    float *Bx;   // (n, P) row-major: candidate j of row i at Bx[i * ldr + j]
    size_t ldr;  // >= P
    double *s;   // [P] squared norms
    double *ybx; // [P]
    double *mom; // [3 P] parent moments (as the SIMT fast pass)
    int *err;    // one int: nonzero when a bounded wait inside a kernel gave up
    void *tab;   // tc_tab_bytes(P): per candidate, its source columns and scale
    double *npart;  // fast_norm_part_bytes(n, P): partial sums of the norms
};

// Largest basis the tensor-core path takes: the T contraction keeps two
// buffers of two 128 x round_up(m, 16) FP32 accumulators in the 512 columns
// of tensor memory.
constexpr int TC_MAX_M = 128;

// Bytes of the per-candidate source table of P candidates.
size_t tc_tab_bytes(size_t P);

// Leading dimensions of the split basis copies for n rows and max_terms columns.
size_t tc_ldn(size_t n);
size_t tc_ldk(size_t max_terms);

// Writes column c of the split copies from the f32 column col (n rows).
void tc_store_column(cudaStream_t st, const float *col, int n, int c, const TcBasis &tb,
                     long long *launches);

// Split-K factor of the tensor-core T contraction for n rows and P candidates.
int tc_ksplit(int n, int P);

// The two-pass projection into row-major Bx, then s = ||Bx||^2,
// ybx = scale(s) (Bx . y) and the parent moments, as fast_project (fast.cuh)
// computes them. src and rsrc are the same candidates (rsrc reading the
// row-major basis copy). Throws mgpu::Error(MARS_GPU_ETIMEOUT) when a bounded
// device wait gave up.
void fast_project_tc(cudaStream_t st, const FillSrc &src, const RowFillSrc &rsrc,
                     const TcBasis &tb, int n, int m, int P, const float *y, double tol,
                     const TcScratch &ws, long long *launches);

// One pass only, for tests: T = Bo^T src and Bx = src - Bo T.
void tc_project_pass(cudaStream_t st, const RowFillSrc &src, const TcBasis &tb, int n, int m,
                     int P, const TcScratch &ws, long long *launches);

}  // namespace mgpu
