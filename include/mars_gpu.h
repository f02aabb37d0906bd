/*
 *  mars_gpu.h -- C ABI of the GB300 MARS forward pass.
 *
 *  Plain C types only (pointers, sizes, status codes): no CUDA or torch types
 *  cross this boundary, and no C++ exception escapes it. Every entry point
 *  returns MARS_GPU_OK (0) or a nonzero status; mars_gpu_last_error() then
 *  holds a message (per calling thread). The fit API takes host arrays and the
 *  library owns its device memory; the kernel-level entry points marked
 *  "DEVICE arrays" take caller-owned device memory and a stream.
 *
 *  A handle is the device-resident state of one fit (the reference's
 *  MarsAlgo plus its mars::cuda::Context). Calls on one handle must not
 *  overlap; different handles may be driven from different threads.
 *
 *  Reference interfaces replaced (file:line in aleon1138/mars):
 *    mars_gpu_create     MarsAlgo::MarsAlgo            marsalgo.cc:266-370
 *                        mars::cuda::context_create    cuda/mars_cuda.h:43
 *                        (+ set_target/sync_xcols      cuda/mars_cuda.h:80,95)
 *    mars_gpu_destroy    MarsAlgo::~MarsAlgo           marsalgo.cc:372-380
 *                        mars::cuda::context_destroy   cuda/mars_cuda.h:48
 *    mars_gpu_nbasis     MarsAlgo::nbasis              marsalgo.h:37
 *    mars_gpu_yvar       MarsAlgo::yvar                marsalgo.h:40
 *    mars_gpu_dsse       MarsAlgo::dsse                marsalgo.h:39
 *    mars_gpu_eval       marslib eval (all X columns)  marslib.cc:41-148
 *                        -> MarsAlgo::eval per column  marsalgo.cc:402-662
 *                        -> MarsAlgo::eval_batch       marsalgo.cc:664-758
 *    mars_gpu_append     MarsAlgo::append              marsalgo.cc:760-875
 *    mars_gpu_orthonormalize   mars::orthonormalize    kernels.h:52-62
 *                              mars::cuda::orthonormalize  cuda/mars_cuda.h:127-131
 *    mars_gpu_orthonormalize_col  mars::orthonormalize_col  kernels.h:91-96
 *    mars_gpu_expand(_backward)   mars.expand (numpy)        mars.py:423-450
 *    mars_gpu_gram                mars.gram (numpy)          mars.py:456-490
 */
#ifndef MARS_GPU_H
#define MARS_GPU_H

#include <stdbool.h>
#include <stddef.h>

#if defined(__GNUC__)
#define MARS_GPU_API __attribute__((visibility("default")))
#else
#define MARS_GPU_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define MARS_GPU_OK 0
#define MARS_GPU_EINVAL 1   /* invalid argument (same messages as the reference) */
#define MARS_GPU_ECUDA 2    /* CUDA runtime / launch failure */
#define MARS_GPU_ENOMEM 3   /* device allocation failed */
#define MARS_GPU_EFULL 4    /* basis matrix is full */
#define MARS_GPU_ETIMEOUT 5 /* a bounded device-side wait ran out */

/* Arithmetic used for candidate evaluation. */
#define MARS_GPU_PREC_FP64 0  /* plain FP64 forward pass */
#define MARS_GPU_PREC_MIXED 1 /* FP32 / FP64-carry fast pass; the best-ranked and the
                                  numerically unreliable candidates re-decided in FP64 */

typedef struct mars_gpu_algo mars_gpu_algo;

typedef struct {
    long long evals;            /* mars_gpu_eval calls */
    long long candidates;       /* (input, parent) pairs evaluated */
    long long knot_evals;       /* grid cuts scored by the hinge sweep */
    long long dgks_fired;       /* candidate columns re-orthogonalised */
    long long redecided;        /* candidates re-evaluated in FP64 (mixed mode) */
    long long kernel_launches;  /* kernels of this library launched by this handle */
    long long h2d_bytes;        /* host-to-device bytes copied by this handle */
    long long d2h_bytes;        /* device-to-host bytes copied by this handle */
    double project_flops;       /* algorithmic projection FLOPs: 4 n m per candidate */
    double sweep_bytes;         /* algorithmic sweep bytes: n (12 + 4 m + 8 P_x) per input */
    double ms_span;             /* device time from the first eval to the last call */
    double ms_project;          /* device time per phase, summed (CUDA events) */
    double ms_dgks;
    double ms_normalize;
    double ms_sweep;
    double ms_sort;
    double ms_append;
    double ms_redecide;         /* mixed mode: wall time of the exact re-decisions */
    double ms_gather;           /* mixed mode: parents and candidates into sorted order */
    double ms_redecide_gpu;     /* mixed mode: device time of re-decisions run on the GPU */
    long long redecided_flagged; /* mixed mode: candidates re-decided for a flag (degenerate
                                    column or unresolvable cut), whatever their rank */
    long long evals_exact;      /* mixed mode: evals run on the exact path after a step that
                                   re-decided most of its candidates */
    long long redecided_degenerate; /* mixed mode: flagged candidates whose projected column
                                       is nearly in the span of the basis */
} mars_gpu_stats;

/* Message of the last failing call on this thread ("" if none). */
MARS_GPU_API const char *mars_gpu_last_error(void);

/* Number of CUDA devices visible (0 when none); never fails. */
MARS_GPU_API int mars_gpu_device_count(void);

/*
 *  Build the fit state. X: (n, p) column-major f32, column stride ldx (>= n);
 *  y, w: (n) f32 (w are inverse-variance weights; non-finite y rows get
 *  weight 0). max_terms: basis capacity including the intercept.
 *  Errors: "target Y is all zero or NANs", "not all columns in X are finite".
 *  X is copied to the device and also borrowed, like the reference's
 *  MarsAlgo borrows it: it must stay valid and unchanged until
 *  mars_gpu_destroy (mars_gpu_eval reads each knot, X[k, i], from it).
 */
MARS_GPU_API int mars_gpu_create(const float *X, const float *y, const float *w, size_t n, size_t p,
                    size_t ldx, size_t max_terms, mars_gpu_algo **out);
MARS_GPU_API int mars_gpu_destroy(mars_gpu_algo *algo);

MARS_GPU_API int mars_gpu_nbasis(const mars_gpu_algo *algo, int *out);
MARS_GPU_API int mars_gpu_yvar(const mars_gpu_algo *algo, double *out);
MARS_GPU_API int mars_gpu_dsse(const mars_gpu_algo *algo, double *out);

/* Select MARS_GPU_PREC_FP64 (the default) or MARS_GPU_PREC_MIXED. */
MARS_GPU_API int mars_gpu_set_precision(mars_gpu_algo *algo, int mode);

/*
 *  Evaluate every (input, parent) pair selected by `mask` in one call.
 *  mask: (rows, nbasis) row-major bool, row stride mask_stride (elements);
 *  rows <= p; row i is input column i. min_span >= 1; end_span rows are
 *  skipped at both ends of the sorted column; linear_only skips the sweep.
 *  Outputs (rows, nbasis) row-major f64, contiguous:
 *    linear[i,j] = delta SSE of adding x_i * B_j
 *    hinge[i,j]  = delta SSE of the best mirror-hinge pair (0 if none)
 *    cut[i,j]    = its knot X[k, i] (NaN if none or linear_only)
 *  sse0 (optional) receives mars_gpu_dsse().
 */
MARS_GPU_API int mars_gpu_eval(mars_gpu_algo *algo, const bool *mask, int rows, int mask_stride,
                  int min_span, int end_span, int linear_only, double *sse0, double *linear,
                  double *hinge, double *cut);

/*
 *  Append basis type 'l' (x * B_bcol), '+' (B_bcol * max(x - h, 0)) or
 *  '-' (B_bcol * max(h - x, 0)) on input xcol. *mse receives the new MSE, or
 *  -1 when the column is numerically degenerate (the basis is unchanged).
 *  Errors: "basis matrix is full", "invalid basis column number: N",
 *  "invalid X column index", "invalid basis type".
 */
MARS_GPU_API int mars_gpu_append(mars_gpu_algo *algo, char type, int xcol, int bcol, float h, double *mse);

/* Counters and per-phase device times of this handle. */
MARS_GPU_API int mars_gpu_get_stats(const mars_gpu_algo *algo, mars_gpu_stats *out);

/*
 *  max |Q^T Q - I| over the live orthonormal basis Q (f32 storage, FP64
 *  arithmetic), and the RSS of the current fit, 1 - sum(ybo^2), recomputed
 *  in FP64 from Q and y.
 */
MARS_GPU_API int mars_gpu_orth_error(mars_gpu_algo *algo, double *max_abs, double *rss);

/*
 *  The same two figures for every leading basis of the fit: entry k (k <
 *  min(cap, m), m = the live basis' size, returned in *count) is max
 *  |Q_k^T Q_k - I| and 1 - sum(ybo^2) over the first k + 1 columns, what the
 *  fit measured when its step reached k + 1 terms (stored columns do not change
 *  after their append). max_abs and rss may be NULL. The last entry equals
 *  mars_gpu_orth_error's pair.
 */
MARS_GPU_API int mars_gpu_orth_error_by_terms(mars_gpu_algo *algo, double *max_abs, double *rss,
                                              size_t cap, size_t *count);

/*
 *  Kernel-level entry points (host arrays in and out), for tests and
 *  micro-benchmarks.
 *
 *  mars_gpu_orthonormalize: for j < p, Bx[:,j] = B[:,mask[j]] * x, project out
 *  the m columns of Bo, DGKS retry when 9 s < ||Bo^T Bx||^2, normalise by
 *  1/sqrt(s+tol) (zero when s <= tol). B: (n, *) column-major, column stride
 *  ldB; Bo: (n, >= m) row-major, row stride ldBo; Bx: (n, p) column-major,
 *  column stride ldBx [out]; s: (p) squared norms before scaling [out,
 *  optional]; dgks: number of columns retried [out, optional].
 */
MARS_GPU_API int mars_gpu_orthonormalize(size_t n, size_t m, size_t p, const float *B, size_t ldB,
                            const float *x, const int *mask, const float *Bo, size_t ldBo,
                            float *Bx, size_t ldBx, double *s, double tol, long *dgks);

/*
 *  mars_gpu_orthonormalize_col: modified Gram-Schmidt of v (n, f64, in/out)
 *  against the m columns of Bo (row-major, stride ldBo) with one DGKS retry;
 *  v is normalised when ||v||^2 > tol. *w receives the pre-normalisation norm.
 */
MARS_GPU_API int mars_gpu_orthonormalize_col(size_t n, size_t m, double *v, const float *Bo, size_t ldBo,
                                double tol, double *w, long *dgks);

/*
 *  Differentiable expansion of a fitted model: the basis of mars.expand
 *  (mars.py:423-450) with the prediction pred = B beta, and its backward pass.
 *  No counterpart in the reference (its expand is numpy, without gradients).
 *
 *  Term j (0 <= j < M, in model order): kind[j] (MARS_GPU_TERM_*), parent[j]
 *  (< j; ignored for the intercept), input[j] (X column), knot[j] (hinges),
 *  beta[j]. B_0 = 1, B_j = B_parent * f_j(x_input), f = x, max(x - t, 0) or
 *  max(t - x, 0). All arrays are DEVICE arrays; X is (N, *) column-major with
 *  column stride ldx; stream is a cudaStream_t (NULL: the default stream).
 *
 *  mars_gpu_expand: pred (N, optional) and B ((N, M) column-major, stride ldb,
 *  optional). mars_gpu_expand_backward: given g = dL/dpred (N), accumulates
 *  dL/dX into dX ((N, *) column-major, stride lddx, optional; the caller zeroes
 *  it) and writes dL/dbeta and dL/dknot (M doubles each; the knot derivative of
 *  a non-hinge term is 0; subgradient 0 at a kink). workspace holds
 *  mars_gpu_expand_workspace(N, M) bytes. 1 <= M <= 128.
 */
#define MARS_GPU_TERM_INTERCEPT 0
#define MARS_GPU_TERM_LINEAR 1
#define MARS_GPU_TERM_PLUS 2
#define MARS_GPU_TERM_MINUS 3
MARS_GPU_API size_t mars_gpu_expand_workspace(size_t N, int M);
MARS_GPU_API int mars_gpu_expand(const int *kind, const int *parent, const int *input,
                    const float *knot, const float *beta, int M, const float *X, size_t ldx,
                    size_t N, float *pred, float *B, size_t ldb, void *stream);
MARS_GPU_API int mars_gpu_expand_backward(const int *kind, const int *parent, const int *input,
                             const float *knot, const float *beta, int M, const float *X,
                             size_t ldx, size_t N, const float *g, float *dX, size_t lddx,
                             double *dbeta, double *dknot, void *workspace, void *stream);

/*
 *  mars_gpu_orthonormalize_noalloc: mars_gpu_orthonormalize on DEVICE arrays,
 *  queued on the caller's stream, allocating no device memory. It has no
 *  counterpart in the reference (its mars::cuda::orthonormalize allocates).
 *
 *  For callers that cannot let a library allocate: a process whose own pool
 *  (for example PyTorch's caching allocator) holds the device memory, so a
 *  cudaMalloc inside the library could fail; and a caller with work running on
 *  other streams, which a cudaFree would stall because it waits for the whole
 *  device.
 *
 *  B, x, Bo, Bx and s are device pointers with the meanings and layouts of
 *  mars_gpu_orthonormalize; B has ncolB columns and every mask[j] must be below
 *  ncolB (checked); mask (p ints) is a host array. s may be NULL. stream is a
 *  cudaStream_t (NULL: the default stream). The working memory is one fixed
 *  array of module-scope device memory (about 2.2 MB per device, held by every
 *  device that loads the library until the process exits), so
 *  p <= MARS_GPU_NOALLOC_MAX_CANDIDATES and m * p <= MARS_GPU_NOALLOC_MAX_COEFS;
 *  larger problems are rejected with MARS_GPU_EINVAL before any work is queued.
 *  The caller clears nothing: every scratch value read is written earlier in
 *  the same call.
 *
 *  Each call looks up the scratch address with the calling thread's current
 *  device (the first call on a device also loads the module there). The call
 *  copies the mask from pageable host memory and synchronises `stream` once
 *  (to read how many columns DGKS retried), so it cannot be issued while that
 *  stream is being captured into a CUDA graph. It returns with the final
 *  scaling queued. All calls on one device share the one scratch array: calls
 *  that overlap -- from two host threads, or on two streams whose work can run
 *  at the same time -- race and give wrong results.
 */
#define MARS_GPU_NOALLOC_MAX_CANDIDATES 4096
#define MARS_GPU_NOALLOC_MAX_COEFS 262144
MARS_GPU_API int mars_gpu_orthonormalize_noalloc(size_t n, size_t m, size_t p, const float *B,
                                    size_t ldB, size_t ncolB, const float *x, const int *mask,
                                    const float *Bo, size_t ldBo, float *Bx, size_t ldBx,
                                    double *s, double tol, void *stream, long *dgks);

/*
 *  mars_gpu_fast_project: the projection of the mixed-precision fast pass, on
 *  host arrays. No counterpart in the reference (whose GPU projection,
 *  mars::cuda::project_reduce at cuda/orthonormalize.cu:704-930, runs on
 *  cuBLAS in blocked f32 or f64): candidate j is v_j = B[:, cand_b[j]] *
 *  (X[:, cand_x[j]] * s[cand_x[j]]) (f32); it is projected onto the
 *  complement of the m columns of Bo ((n, m) column-major, stride ldBo):
 *  T = Bo^T v, Bx = v - Bo T. passes = 2 applies it twice (the second pass on
 *  the first one's residual) and fills s_out = ||Bx||^2 and
 *  ybx_out = (Bx . y) / sqrt(s + tol) (both optional); passes = 1 stops after
 *  one. T (P x m, row j = candidate j) receives the last pass's coefficients,
 *  Bx (n x P row-major, candidate j of row i at Bx[i P + j], the layout the
 *  fast hinge sweep reads) the projected columns. use_tc = 1: the
 *  tensor-core kernels (tcgen05, split-TF32; m <= 128); use_tc = 0: the FP32
 *  SIMT kernels (passes = 2 only). ms_out (optional) receives the device time
 *  of the projection kernels (CUDA events on the call's stream), copies
 *  excluded.
 */
MARS_GPU_API int mars_gpu_fast_project(size_t n, size_t m, size_t P, const float *B, size_t ldB,
                                       size_t ncolB, const float *X, size_t ldX, size_t ncolX,
                                       const float *s, const int *cand_x, const int *cand_b,
                                       const float *Bo, size_t ldBo, const float *y, double tol,
                                       int use_tc, int passes, float *T, float *Bx,
                                       double *s_out, double *ybx_out, float *ms_out);

/*
 *  mars_gpu_gram: out (ka x kb, row-major) = A^T B for A (n, ka) and B (n, kb)
 *  column-major f32 host arrays (column strides lda, ldb >= n), in the
 *  arithmetic of mars.gram (mars.py:456-490): per 128-row chunk a fused
 *  multiply-add chain in f32 over the rows in order, the chunk results added
 *  in float64 in chunk order. exact = 1 instead widens every product exactly
 *  and runs the chunk chains in FP64 (for the matrix-vector products, which
 *  the reference's BLAS forms in another order). The Gram matrices of the
 *  backward pass (mars.prune, mars.py:622-695).
 */
MARS_GPU_API int mars_gpu_gram(size_t n, const float *A, size_t lda, size_t ka, const float *B,
                               size_t ldb, size_t kb, int exact, double *out);
/* The same for float64 inputs (the chunk chains in float64). */
MARS_GPU_API int mars_gpu_gram_f64(size_t n, const double *A, size_t lda, size_t ka,
                                   const double *B, size_t ldb, size_t kb, int exact,
                                   double *out);

/*
 *  Bytes currently handed out by the library's stream-ordered memory pool on
 *  the calling thread's current device (cudaMemPoolAttrUsedMemCurrent): what
 *  live handles hold. A diagnostic for tests (a call that allocates nothing
 *  leaves it unchanged); never fails when a device is visible.
 */
MARS_GPU_API int mars_gpu_pool_used_bytes(size_t *out);


#ifdef __cplusplus
}
#endif

#endif /* MARS_GPU_H */
