// FP64 forward-pass kernels: the plain FP64 GPU path and the FP64 re-decision
// path of the mixed mode. Launch wrappers are host functions on a stream.
#pragma once

#include "common.cuh"
#include "xappend.cuh"

namespace mgpu {

// Candidate column source: Bx[i, j] = B[i, cand_b[j]] * (X[i, cand_x[j]] * s[cand_x[j]]),
// both products in f32 (marsalgo.cc:436-441 and kernels.cc:298-312).
struct FillSrc {
    const float *B;
    size_t ldB;
    const float *X;
    size_t ldX;
    const float *s;
    const int *cand_x;
    const int *cand_b;
    __device__ __forceinline__ float operator()(size_t i, int j) const
    {
        const int xc = cand_x[j];
        return B[i + (size_t)cand_b[j] * ldB] * (X[i + (size_t)xc * ldX] * s[xc]);
    }
    // The same value from its raw columns: combine(B[i, cand_b[j]], X[i, cand_x[j]], s[cand_x[j]]).
    static constexpr int kRaw = 2;
    __device__ __forceinline__ const float *raw0(int j) const { return B + (size_t)cand_b[j] * ldB; }
    __device__ __forceinline__ const float *raw1(int j) const { return X + (size_t)cand_x[j] * ldX; }
    __device__ __forceinline__ float param(int j) const { return s[cand_x[j]]; }
    __device__ __forceinline__ static float combine(float b, float x, float sx) { return b * (x * sx); }
    // element strides of raw0 / raw1 from one row to the next
    __host__ __device__ static constexpr size_t stride0() { return 1; }
    __host__ __device__ static constexpr size_t stride1() { return 1; }
};

// FillSrc with the basis read from a row-major copy BR (n, ldBR): the same
// value, B[i, b] * (X[i, x] * s[x]), for kernels whose warps cover several
// candidates of one row (their parents then lie in one row of BR).
struct RowFillSrc {
    const float *BR;
    size_t ldBR;
    const float *X;
    size_t ldX;
    const float *s;
    const int *cand_x;
    const int *cand_b;
    __device__ __forceinline__ float operator()(size_t i, int j) const
    {
        const int xc = cand_x[j];
        return BR[i * ldBR + cand_b[j]] * (X[i + (size_t)xc * ldX] * s[xc]);
    }
    static constexpr int kRaw = 2;
    __device__ __forceinline__ const float *raw0(int j) const { return BR + cand_b[j]; }
    __device__ __forceinline__ const float *raw1(int j) const { return X + (size_t)cand_x[j] * ldX; }
    __device__ __forceinline__ float param(int j) const { return s[cand_x[j]]; }
    __device__ __forceinline__ static float combine(float b, float x, float sx) { return b * (x * sx); }
    __host__ __device__ size_t stride0() const { return ldBR; }
    __host__ __device__ static constexpr size_t stride1() { return 1; }
};

// Candidate columns stored row-major: Bx[i * ldr + j] (the mixed fast pass's
// layout, so that a row's candidates are contiguous for the hinge sweep).
struct RowStoredSrc {
    const float *Bx;
    size_t ldr;
    __device__ __forceinline__ float operator()(size_t i, int j) const { return Bx[i * ldr + j]; }
    static constexpr int kRaw = 1;
    __device__ __forceinline__ const float *raw0(int j) const { return Bx + j; }
    __device__ __forceinline__ const float *raw1(int j) const { return Bx + j; }
    __device__ __forceinline__ float param(int) const { return 0.f; }
    __device__ __forceinline__ static float combine(float v, float, float) { return v; }
    __host__ __device__ size_t stride0() const { return ldr; }
    __host__ __device__ size_t stride1() const { return ldr; }
};

// Candidate column source: an already-stored f32 column Bx[:, col[j]] (col may be null).
struct StoredSrc {
    const float *Bx;
    size_t ldBx;
    const int *col;
    __device__ __forceinline__ float operator()(size_t i, int j) const
    {
        const int c = col ? col[j] : j;
        return Bx[i + (size_t)c * ldBx];
    }
    static constexpr int kRaw = 1;
    __device__ __forceinline__ const float *raw0(int j) const
    {
        return Bx + (size_t)(col ? col[j] : j) * ldBx;
    }
    __device__ __forceinline__ const float *raw1(int j) const { return raw0(j); }
    __device__ __forceinline__ float param(int) const { return 0.f; }
    __device__ __forceinline__ static float combine(float v, float, float) { return v; }
    __host__ __device__ static constexpr size_t stride0() { return 1; }
    __host__ __device__ static constexpr size_t stride1() { return 1; }
};

// One block of the hinge sweep: up to 8 candidates that share an input column.
struct SweepTask {
    int xcol;
    int cand0;
    int count;
};

// Projection of P candidate columns onto the m columns of Bo (row-major, ldbo).
//   T = Bo^T Bx               (FP64 accumulation, deterministic split-K)
//   Bx <- f32(Bx - Bo T)      (FP64 arithmetic, one rounding)
//   s  = ||Bx||^2             (FP64, of the rounded values)
// `out_col` maps candidate j to its output column (null: identity).
struct ProjectScratch {
    double *T;  // [P][m]
};

// Bo may be stored as f64 (the fit state) or f32 (the kernel-level entry points).
// BoC and xa, when given, are the same basis as f32 columns (column stride n)
// and scratch: with few entries (P m, a DGKS re-pass over stored columns) T is
// then formed by the exact parallel chains of tgemm_exact (xappend.cuh), which
// give the values of the chains run in order.
template <class Src, class BoT>
void project_fp64(cudaStream_t st, const Src &src, const BoT *Bo, size_t ldbo, const float *BoC,
                  XaBufs *xa, int n, int m, int P, const int *out_col, float *Bx, size_t ldBx,
                  double *s_out, const ProjectScratch &ws, long long *launches);

// T[j][c] = sum_i Bo[i,c] * src(i, j) only, each entry one fused chain over
// the rows in order (the reference's accumulation order).
template <class Src, class BoT>
void tgemm_fp64(cudaStream_t st, const Src &src, const BoT *Bo, size_t ldbo, int n, int m,
                int P, double *T, long long *launches);

// s[fired[q]] = snew[q] for q < nf.
void scatter_s(cudaStream_t st, const int *fired, int nf, const double *snew, double *s,
               long long *launches);

// DGKS gate (kernels.cc:384-395): fired = s > tol && 9 s < ||T_j||^2; the
// fired candidate indexes are appended to `fired` (count in *nfired).
void dgks_gate(cudaStream_t st, const double *T, int m, int P, const double *s, double tol,
               int *fired, int *nfired, long long *launches);

// Normalise (kernels.cc:401-416) and ybx = Bx^T y (kernels.cc:215-237):
// scale = s > tol ? f32(1/sqrt(s+tol)) : 0; Bx *= scale (if store); ybx in FP64.
void normalize_ybx(cudaStream_t st, float *Bx, size_t ldBx, int n, int P, const double *s,
                   double tol, const float *y, bool store, double *ybx, long long *launches);

// Bx[:, j] *= scale(s[j]) for j < P, the scaling step of normalize_ybx alone.
void scale_columns(cudaStream_t st, float *Bx, size_t ldBx, int n, int P, const double *s,
                   double tol, long long *launches);

// Candidates per hinge-sweep block for m live basis columns and `candidates`
// candidates in the launch (sweep_split warps each).
int sweep_warps(int m, int candidates);

// Number of grid rows (cut candidates) of the sweep: rows head+1, head+1+min_span, ... < tail.
int sweep_grid_rows(int head, int tail, int min_span);

// The sweep's inputs in the descending order of each candidate's input
// column: bs[j * n + i] = B[perm_x[i], cand_b[j]] and bxs[j * n + i] =
// f32(Bx[perm_x[i], j] * scale_j), for sorted rows i < rows.
void gather_parents(cudaStream_t st, const int *perm, const float *B, size_t ldB,
                    const int *cand_x, const int *cand_b, int n, int rows, int P, float *bs,
                    long long *launches);
void gather_candidates(cudaStream_t st, const int *perm, const float *Bx, size_t ldBx,
                       const int *cand_x, const double *s, double tol, int n, int rows, int P,
                       float *bxs, long long *launches);

// Scalar recurrences of the hinge sweep (k0, k1, w at every grid row) for the
// candidates of `tasks` (at most 32 per task, one input column each), from the
// sorted parents bs and the sorted y; scal holds (candidates,
// sweep_grid_rows, 3) doubles. ncand: the candidates of all tasks together.
void hinge_scalars(cudaStream_t st, const SweepTask *tasks, int ntasks, int ncand,
                   const float *xsort, const float *ysort, const float *bs, int n, int head,
                   int tail, int min_span, double *scal, long long *launches);

// Hinge sweep in FP64 (marsalgo.cc:508-657), one warp per candidate; tasks
// hold at most sweep_warps(m) candidates; scal from hinge_scalars.
// With part == nullptr it scores the cuts with ybx and writes hsse/hrow.
// Otherwise ybx is not read: per candidate j and grid row g it stores
// part[(j * ngrid + g) * 4 + {0..3}] = {fy before its last step (the
// candidate component's), f_m, w, den}, and sweep_score finishes the scores
// once ybx is known -- so the sweep need not wait for the ybx chain.
void sweep_fp64(cudaStream_t st, const SweepTask *tasks, int ntasks, const int *perm,
                const float *xsort, const float *bs, const float *bxs, const double *Bo,
                size_t ldbo, const double *ybo, const double *ybx, const double *scal, int n,
                int m, int head, int tail, int min_span, double tol, double *hsse, int *hrow,
                int warps_per_block, long long *launches, double *part = nullptr,
                int split = 1);

// Warps per candidate of the FP64 sweep (1 or 2) for m basis columns and
// `candidates` candidates in the launch; sweep_warps already accounts for it.
int sweep_split(int m, int candidates);

// The scores of the deferred sweep (the reference's: fy = fy_partial + f_m ybx
// as the chain's last fused step, uw = fy - w, sse = den > tol ? uw^2 / (den +
// tol) : 0) and the first maximum in row order, for candidates j < P (input
// cand_x[j]).
void sweep_score(cudaStream_t st, const double *part, int P, const int *cand_x,
                 const int *perm, const double *ybx, int n, int head, int tail, int min_span,
                 double tol, double *hsse, int *hrow, long long *launches);

// Stable descending argsort of X columns (marsalgo.cc:33-39), the scaled
// sorted values xsort[i] = X[perm[i]] * s and the sorted target ysort[i] = y[perm[i]].
void sort_columns(cudaStream_t st, const float *X, size_t ldX, const float *s, const float *y,
                  int n, const int *cols, int ncols, int *perm, float *xsort, float *ysort,
                  DevBuf &keys, DevBuf &vals, DevBuf &tmp, long long *launches);

// Scatter per-candidate results into the (rows, m) outputs.
void assemble_outputs(cudaStream_t st, int P, const int *cand_x, const int *cand_b, int m,
                      const double *ybx, const double *hsse, const int *hrow, const float *X,
                      size_t ldX, bool linear_only, double *lin, double *hin, double *cut,
                      long long *launches);
void fill_outputs(cudaStream_t st, int rows, int m, double *lin, double *hin, double *cut,
                  long long *launches);

// Column sums of squares sum_i X[i,j]^2 in FP64 (for s = 1/rms).
void column_sumsq(cudaStream_t st, const float *X, size_t ldX, int n, int p, double *out,
                  long long *launches);


}  // namespace mgpu
