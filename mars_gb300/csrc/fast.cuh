// Fast (ranking) pass of the mixed-precision forward pass: every candidate
// scored in FP32 with FP64 carries; the decisions are then re-taken from the
// exact FP64 values of the best-ranked candidates (host_exact.h).
#pragma once

#include "common.cuh"
#include "fp64.cuh"

#include <vector>

namespace mgpu {

struct FastScratch {
    float *Tp;     // split-K partial T: [ksplit][P][m]
    float *T;      // [P][m]
    float *Bx;     // projected candidate columns, (n, P) column-major, ld n
    double *s;     // [P] squared norms of the projected columns
    double *ybx;   // [P] y . normalised column
    double *mom;   // [3 P] sum b^2 x^k, k = 0..2 (parent b, input x); k = 2: raw norm of x b
};

// Split-K factor of the fast projection for n rows.
int fast_ksplit(int n);

// Bx = v - Bo (Bo^T v) twice (the second pass re-orthogonalises the residual
// of the first), v = src (FillSrc), then s = ||Bx||^2 and
// ybx = scale(s) * (Bx . y), and the parent moments mom. BoC: (n, m) column-major f32 (ld n).
void fast_project(cudaStream_t st, const FillSrc &src, const float *BoC, int n, int m, int P,
                  const float *y, double tol, const FastScratch &ws, long long *launches);

// s = ||Bx||^2, ybx = scale(s) (Bx . y) and the parent moments mom (the last
// steps of fast_project).
void fast_norms_moments(cudaStream_t st, const float *Bx, int n, const float *y, double tol,
                        const FillSrc &src, int P, double *s, double *ybx, double *mom,
                        long long *launches);

// s and ybx (as fast_norms_moments) of row-major candidate columns Bx (ld
// ldr); part holds fast_norm_part_bytes(n, P) of partial sums.
size_t fast_norm_part_bytes(size_t n, size_t P);
void fast_norms_rows(cudaStream_t st, const float *Bx, size_t ldr, int n, const float *y,
                     double tol, int P, double *part, double *s, double *ybx,
                     long long *launches);
// The parent moments alone (the last step of fast_norms_moments).
void fast_parent_moments(cudaStream_t st, const FillSrc &src, int n, int P, double *mom,
                         long long *launches);
// Column-major candidate columns (ld n) to the row-major layout (ld ldr).
void fast_to_rows(cudaStream_t st, const float *Bc, int n, int P, float *Br, size_t ldr,
                  long long *launches);

// Chunked FP32 / FP64-carry hinge sweep of every candidate, in two halves:
// tasks with dir 0 sweep from the top and score the cuts up to
// fast_sweep_mid(), tasks with dir 1 sweep the mirror hinge from the bottom
// and score the rest. Outputs per candidate j and direction:
// hsse[2 j + dir] (the hinge part of the best score), hrow[2 j + dir], and
// hflag[2 j + dir] = 1 when a cut of that half has den below cut_rel of the
// reference's K (its f64 value there is unreliable). mom: from fast_project.
// `tasks` are SweepTask-sized records {xcol, cand0, count, dir}; BoR: (n, ldbo)
// row-major f32 basis (ldbo a multiple of 4).
int fast_sweep_warps(int m, const std::vector<int> &group_sizes);  // candidates per input column
// The sweep's per-candidate columns, read in each input's sorted order by the
// sweep itself, both row-major so that a sorted row's values for the block's
// candidates share one or two memory sectors: the parent BR[i * ldBR +
// cand_b[j]] (the row-major copy of the basis) and the projected candidate
// Bx[i * ldr + j], normalised there by f32(1 / sqrt(s[j] + tol)).
struct FastSweepCols {
    const float *BR;
    size_t ldBR;
    const int *cand_b;
    const float *Bx;
    size_t ldr;
    const double *s;
};
int fast_sweep_mid(int head, int tail, int n);  // in [0, n - 1]
struct FastTaskRec {
    int xcol, cand0, count, dir;
};
void fast_sweep(cudaStream_t st, const FastTaskRec *tasks, int ntasks, const int *perm,
                const float *xsort, const float *ysort, const FastSweepCols &cols,
                const float *BoR, size_t ldbo, const double *ybo, const double *ybx,
                const double *mom, int n, int m, int head, int tail, int min_span, double tol,
                double cut_rel, double *hsse, int *hrow, int *hflag, int warps_per_block,
                long long *launches);

}  // namespace mgpu
