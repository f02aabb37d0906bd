// FP64 forward-pass kernels (the plain FP64 GPU path; also the re-decision
// path of the mixed mode). Arithmetic follows the reference CPU path
// operation for operation where the order is local (per element, per
// candidate); long reductions over rows are split deterministically
// (fixed per-thread order, fixed block tree, fixed order across blocks).
#include "fp64.cuh"

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

namespace mgpu {
namespace {

// ---------------------------------------------------------------------------
// T = Bo^T Bx, split over rows (K). Block tile: 64 components x 32 columns,
// 32 rows per stage. Each thread owns one component and 8 columns.
// ---------------------------------------------------------------------------
constexpr int TG_ROWS = 32, TG_COMPS = 64, TG_COLS = 32, TG_THREADS = 256;

template <class Src>
__global__ void __launch_bounds__(TG_THREADS)
    k_tgemm(Src src, const float *__restrict__ Bo, size_t ldbo, int n, int m, int P,
            int rows_per_split, double *__restrict__ Tpart)
{
    __shared__ float sBo[TG_ROWS][TG_COMPS + 1];
    __shared__ float sV[TG_ROWS][TG_COLS + 1];
    const int t = threadIdx.x, cl = t & (TG_COMPS - 1), jg = t / TG_COMPS;
    const int col0 = blockIdx.x * TG_COLS, split = blockIdx.y, c0 = blockIdx.z * TG_COMPS;
    const size_t rb = (size_t)split * rows_per_split;
    const size_t re = min((size_t)n, rb + (size_t)rows_per_split);
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        acc[q] = 0.0;
    }
    for (size_t r0 = rb; r0 < re; r0 += TG_ROWS) {
        for (int e = t; e < TG_ROWS * TG_COMPS; e += TG_THREADS) {
            const int rr = e / TG_COMPS, cc = e % TG_COMPS;
            const size_t i = r0 + rr;
            const int c = c0 + cc;
            sBo[rr][cc] = (i < re && c < m) ? Bo[i * ldbo + c] : 0.f;
        }
        for (int e = t; e < TG_ROWS * TG_COLS; e += TG_THREADS) {
            const int rr = e % TG_ROWS, jj = e / TG_ROWS;
            const size_t i = r0 + rr;
            const int col = col0 + jj;
            sV[rr][jj] = (i < re && col < P) ? src(i, col) : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int rr = 0; rr < TG_ROWS; ++rr) {
            const double bo = (double)sBo[rr][cl];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                acc[q] = fma(bo, (double)sV[rr][jg * 8 + q], acc[q]);
            }
        }
        __syncthreads();
    }
    const int c = c0 + cl;
    if (c < m) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int col = col0 + jg * 8 + q;
            if (col < P) {
                Tpart[((size_t)split * P + col) * m + c] = acc[q];
            }
        }
    }
}

__global__ void k_reduce_splits(const double *__restrict__ part, int splits, size_t count,
                                double *__restrict__ out)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count) {
        return;
    }
    double s = part[idx];
    for (int sp = 1; sp < splits; ++sp) {
        s += part[(size_t)sp * count + idx];
    }
    out[idx] = s;
}

// out[j] = sum_b part[b*P + j] in block order.
__global__ void k_reduce_cols(const double *__restrict__ part, int nb, int P,
                              double *__restrict__ out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= P) {
        return;
    }
    double s = 0.0;
    for (int b = 0; b < nb; ++b) {
        s += part[(size_t)b * P + j];
    }
    out[j] = s;
}

// ---------------------------------------------------------------------------
// Bx <- f32(Bx - Bo T) per row and candidate; per-block partial ||Bx||^2.
// The projection is the reference's sequential fused chain over k
// (kernels.cc:56-78, 86-118 scalar branches).
// ---------------------------------------------------------------------------
constexpr int PJ_THREADS = 128, PJ_COLS = 8;

template <class Src>
__global__ void __launch_bounds__(PJ_THREADS)
    k_project(Src src, const float *__restrict__ Bo, size_t ldbo, int n, int m, int P,
              const double *__restrict__ T, const int *__restrict__ out_col,
              float *__restrict__ Bx, size_t ldBx, double *__restrict__ part)
{
    extern __shared__ double sT[];  // PJ_COLS * m
    __shared__ double red[32];
    const int t = threadIdx.x, j0 = blockIdx.y * PJ_COLS;
    for (int e = t; e < PJ_COLS * m; e += PJ_THREADS) {
        const int q = e / m, k = e % m, j = j0 + q;
        sT[e] = (j < P) ? T[(size_t)j * m + k] : 0.0;
    }
    __syncthreads();
    const size_t i = (size_t)blockIdx.x * PJ_THREADS + t;
    const float *bo = Bo + (i < (size_t)n ? i : 0) * ldbo;
    for (int q = 0; q < PJ_COLS; ++q) {
        const int j = j0 + q;
        if (j >= P) {
            break;  // uniform over the block
        }
        double sq = 0.0;
        if (i < (size_t)n) {
            double proj = 0.0;
            const double *tj = sT + q * m;
            for (int k = 0; k < m; ++k) {
                proj = fma((double)bo[k], tj[k], proj);
            }
            const double v = (double)src(i, j) - proj;
            const float vf = (float)v;
            const int oc = out_col ? out_col[j] : j;
            Bx[i + (size_t)oc * ldBx] = vf;
            sq = (double)vf * (double)vf;
        }
        const double bs = block_sum<PJ_THREADS>(sq, red);
        if (t == 0) {
            part[(size_t)blockIdx.x * P + j] = bs;
        }
    }
}

__global__ void k_gate(const double *__restrict__ T, int m, int P, const double *__restrict__ s,
                       double tol, int *__restrict__ fired, int *__restrict__ nfired)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= P) {
        return;
    }
    double tn = 0.0;
    for (int k = 0; k < m; ++k) {
        const double v = T[(size_t)j * m + k];
        tn = fma(v, v, tn);
    }
    const double sj = s[j];
    if (sj > tol && sj * 9.0 < tn) {
        const int slot = atomicAdd(nfired, 1);
        fired[slot] = j;
    }
}

// Scatter s of the retried columns: s[fired[q]] = s_new[q].
__global__ void k_scatter_s(const int *__restrict__ fired, int nf, const double *__restrict__ snew,
                            double *__restrict__ s)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nf) {
        s[fired[q]] = snew[q];
    }
}

constexpr int NM_THREADS = 256, NM_COLS = 8;

__global__ void __launch_bounds__(NM_THREADS)
    k_normalize(float *__restrict__ Bx, size_t ldBx, int n, int P, const double *__restrict__ s,
                double tol, const float *__restrict__ y, bool store, double *__restrict__ part)
{
    __shared__ float sc[NM_COLS];
    __shared__ double red[32];
    const int t = threadIdx.x, j0 = blockIdx.y * NM_COLS;
    if (t < NM_COLS) {
        const int j = j0 + t;
        const double sj = j < P ? s[j] : 0.0;
        sc[t] = (sj > tol) ? (float)(1.0 / sqrt(sj + tol)) : 0.0f;
    }
    __syncthreads();
    const size_t i = (size_t)blockIdx.x * NM_THREADS + t;
    const float yi = i < (size_t)n ? y[i] : 0.f;
    for (int q = 0; q < NM_COLS; ++q) {
        const int j = j0 + q;
        if (j >= P) {
            break;
        }
        double prod = 0.0;
        if (i < (size_t)n) {
            const float v = Bx[i + (size_t)j * ldBx] * sc[q];
            if (store) {
                Bx[i + (size_t)j * ldBx] = v;
            }
            prod = (double)v * (double)yi;
        }
        const double bs = block_sum<NM_THREADS>(prod, red);
        if (t == 0) {
            part[(size_t)blockIdx.x * P + j] = bs;
        }
    }
}

// ---------------------------------------------------------------------------
// FP64 hinge sweep (marsalgo.cc:576-649 with covariates_impl :91-151).
// One warp per candidate; lanes own components c = lane + 32 q of f and g
// (component m is the candidate column Bx itself). The sorted rows are staged
// 32 at a time: permutation, deltas, y, the gathered Bo rows (shared by all
// candidates of the block's input column), and per warp B and Bx.
// ---------------------------------------------------------------------------
constexpr int SW_ROWS = 32, SW_WARPS = 8, SW_THREADS = SW_WARPS * 32;

template <int CPL>
__global__ void __launch_bounds__(SW_THREADS)
    k_sweep(const SweepTask *__restrict__ tasks, const int *__restrict__ perm,
            const float *__restrict__ xsort, const float *__restrict__ y,
            const float *__restrict__ B, size_t ldB, const int *__restrict__ cand_b,
            const float *__restrict__ Bx, size_t ldBx, const float *__restrict__ Bo,
            size_t ldbo, const double *__restrict__ ybo, const double *__restrict__ ybx, int n,
            int m, int head, int tail, int min_span, double tol, double *__restrict__ hsse,
            int *__restrict__ hrow)
{
    extern __shared__ float sBo[];  // SW_ROWS * ldS
    __shared__ int sk[SW_ROWS];
    __shared__ float sd[SW_ROWS], sy[SW_ROWS];
    __shared__ float sb[SW_WARPS][SW_ROWS], sbx[SW_WARPS][SW_ROWS];
    const int ldS = m | 1;
    const SweepTask task = tasks[blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool active = warp < task.count;
    const int cand = task.cand0 + (active ? warp : 0);
    const int *pk = perm + (size_t)task.xcol * n;
    const float *xs = xsort + (size_t)task.xcol * n;
    const float *bcol = B + (size_t)cand_b[cand] * ldB;
    const float *bxcol = Bx + (size_t)cand * ldBx;

    double f[CPL], g[CPL], yc[CPL];
#pragma unroll
    for (int q = 0; q < CPL; ++q) {
        const int c = lane + 32 * q;
        f[q] = 0.0;
        g[q] = 0.0;
        yc[q] = c < m ? ybo[c] : (c == m ? ybx[cand] : 0.0);
    }
    double k0 = 0, k1 = 0, w = 0, bd = 0, vb = 0, b2 = 0;
    double best = 0.0;
    int besti = -1;
    long next_grid = (long)head + 1;

    for (int i0 = 0; i0 < tail; i0 += SW_ROWS) {
        const int rows = min(SW_ROWS, tail - i0);
        if (threadIdx.x < rows) {
            const int r = threadIdx.x, i = i0 + r;
            const int k = pk[i];
            sk[r] = k;
            sy[r] = y[k];
            sd[r] = i > 0 ? xs[i - 1] - xs[i] : 0.f;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < rows * m; e += SW_THREADS) {
            const int r = e / m, c = e % m;
            sBo[r * ldS + c] = Bo[(size_t)sk[r] * ldbo + c];
        }
        if (active && lane < rows) {
            sb[warp][lane] = bcol[sk[lane]];
            sbx[warp][lane] = bxcol[sk[lane]];
        }
        __syncthreads();
        if (active) {
            for (int r = 0; r < rows; ++r) {
                const int i = i0 + r;
                const double bk = sb[warp][r], bxk = sbx[warp][r], yk = sy[r];
                const float *row = sBo + r * ldS;
                if (i == 0) {
                    // covariates_impl<false>(.., k0 = 0, k1 = b_k): g = b_k * row.
#pragma unroll
                    for (int q = 0; q < CPL; ++q) {
                        const int c = lane + 32 * q;
                        const double xv = c < m ? (double)row[c] : (c == m ? bxk : 0.0);
                        f[q] = fma(0.0, g[q], f[q]);
                        g[q] = fma(bk, xv, g[q]);
                    }
                    vb = bk * yk;
                    b2 = bk * bk;
                    continue;
                }
                const double di = (double)sd[r];
                const bool on_grid = (i == next_grid);
                if (on_grid) {
                    next_grid += min_span;
                }
                double pf = 0.0, py = 0.0;
#pragma unroll
                for (int q = 0; q < CPL; ++q) {
                    const int c = lane + 32 * q;
                    const double xv = c < m ? (double)row[c] : (c == m ? bxk : 0.0);
                    f[q] = fma(di, g[q], f[q]);
                    g[q] = fma(bk, xv, g[q]);
                    if (on_grid) {
                        pf = fma(f[q], f[q], pf);
                        py = fma(f[q], yc[q], py);
                    }
                }
                k0 = fma(di * di, b2, k0);
                k1 = fma(di * 2, bd, k1);
                w = fma(di, vb, w);
                bd = fma(di, b2, bd);
                b2 = fma(bk, bk, b2);
                vb = fma(yk, bk, vb);
                if (on_grid) {
                    const double ff = warp_sum(pf);
                    const double fy = warp_sum(py);
                    const double uw = fy - w;
                    const double den = (k0 + k1) - ff;
                    const double sse = den > tol ? (uw * uw) / (den + tol) : 0.0;
                    if (sse > best) {
                        best = sse;
                        besti = i;
                    }
                }
            }
        }
        __syncthreads();
    }
    if (active && lane == 0) {
        hsse[cand] = best;
        hrow[cand] = besti >= 0 ? pk[besti] : -1;
    }
}

__global__ void k_sort_keys(const float *__restrict__ X, size_t ldX, int n, int col,
                            float *__restrict__ keys, int *__restrict__ vals)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float x = X[i + (size_t)col * ldX];
        keys[i] = (x == 0.0f) ? 0.0f : x;  // -0 and +0 compare equal in the reference
        vals[i] = i;
    }
}

__global__ void k_gather_scaled(const float *__restrict__ X, size_t ldX, const float *__restrict__ s,
                                int n, int col, const int *__restrict__ perm,
                                float *__restrict__ xsort)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        xsort[i] = X[perm[i] + (size_t)col * ldX] * s[col];
    }
}

__global__ void k_fill_outputs(size_t count, double *lin, double *hin, double *cut)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) {
        lin[i] = 0.0;
        hin[i] = 0.0;
        cut[i] = __longlong_as_double(0x7ff8000000000000LL);
    }
}

__global__ void k_assemble(int P, const int *__restrict__ cx, const int *__restrict__ cb, int m,
                           const double *__restrict__ ybx, const double *__restrict__ hsse,
                           const int *__restrict__ hrow, const float *__restrict__ X, size_t ldX,
                           bool linear_only, double *lin, double *hin, double *cut)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= P) {
        return;
    }
    const size_t idx = (size_t)cx[j] * m + cb[j];
    const double l = ybx[j] * ybx[j];
    lin[idx] = l;
    if (!linear_only && hrow[j] >= 0) {
        hin[idx] = l + hsse[j];
        cut[idx] = (double)X[(size_t)hrow[j] + (size_t)cx[j] * ldX];
    }
}

// ---------------------------------------------------------------------------
// Append: each block owns a contiguous row range; partial sums are reduced in
// block order by every block that needs them (no atomics, deterministic).
// ---------------------------------------------------------------------------
constexpr int AP_THREADS = 256;

__device__ __forceinline__ void block_rows(int n, int nb, int b, int &lo, int &hi)
{
    const int per = (n + nb - 1) / nb;
    lo = min(n, b * per);
    hi = min(n, lo + per);
}

__device__ __forceinline__ double sum_parts(const double *part, int nb)
{
    double s = 0.0;
    for (int b = 0; b < nb; ++b) {
        s += part[b];
    }
    return s;
}

__global__ void __launch_bounds__(AP_THREADS)
    k_append_fill(char type, const float *__restrict__ X, size_t ldX, const float *__restrict__ s,
                  int xcol, float *__restrict__ B, size_t ldB, int bcol, int m, float h, int n,
                  double *__restrict__ v, double *__restrict__ part)
{
    __shared__ double red[32];
    int lo, hi;
    block_rows(n, gridDim.x, blockIdx.x, lo, hi);
    const float sx = s[xcol];
    double acc = 0.0;
    for (int i = lo + threadIdx.x; i < hi; i += AP_THREADS) {
        const float xp = X[(size_t)i + (size_t)xcol * ldX];
        const float bp = B[(size_t)i + (size_t)bcol * ldB];
        float val;
        if (type == 'l') {
            val = sx * bp * xp;
        } else {
            const float t = (type == '+') ? xp - h : h - xp;
            val = sx * bp * ((t < 0.0f) ? 0.0f : t);  // std::max(t, 0.0f)
        }
        B[(size_t)i + (size_t)m * ldB] = val;
        const double vd = (double)val;
        v[i] = vd;
        acc = fma(vd, vd, acc);
    }
    const double bs = block_sum<AP_THREADS>(acc, red);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = bs;
    }
}

__global__ void __launch_bounds__(AP_THREADS)
    k_append_scale(float *__restrict__ B, size_t ldB, int m, int n, const double *__restrict__ part,
                   int nb)
{
    int lo, hi;
    block_rows(n, gridDim.x, blockIdx.x, lo, hi);
    const float raw = (float)sqrt(sum_parts(part, nb));
    for (int i = lo + threadIdx.x; i < hi; i += AP_THREADS) {
        B[(size_t)i + (size_t)m * ldB] /= raw;
    }
}

// Step j of modified Gram-Schmidt: apply coefficient j-1 (reduced from the
// previous step's partials), then the partial dot of column j with v
// (or of v with itself when j == m).
__global__ void __launch_bounds__(AP_THREADS)
    k_mgs_step(const float *__restrict__ BoC, int n, int m, int j, double *__restrict__ v,
               double *__restrict__ part, int nb, double *__restrict__ coef)
{
    __shared__ double red[32];
    int lo, hi;
    block_rows(n, gridDim.x, blockIdx.x, lo, hi);
    double c = 0.0;
    if (j > 0) {
        c = sum_parts(part + ((j - 1) & 1) * nb, nb);
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            coef[j - 1] = c;
        }
    }
    const float *prev = BoC + (size_t)(j > 0 ? j - 1 : 0) * n;
    const float *cur = BoC + (size_t)(j < m ? j : 0) * n;
    double acc = 0.0;
    for (int i = lo + threadIdx.x; i < hi; i += AP_THREADS) {
        double vi = v[i];
        if (j > 0) {
            vi = fma(-c, (double)prev[i], vi);
            v[i] = vi;
        }
        if (j < m) {
            acc = fma((double)cur[i], vi, acc);
        } else {
            acc = fma(vi, vi, acc);
        }
    }
    const double bs = block_sum<AP_THREADS>(acc, red);
    if (threadIdx.x == 0) {
        part[(j & 1) * nb + blockIdx.x] = bs;
    }
}

// scal[0] = sum_j c_j^2 (sequential fused chain), scal[1] = ||v||^2.
__global__ void k_mgs_finish(const double *__restrict__ part, int nb, int m,
                             const double *__restrict__ coef, double *__restrict__ scal)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double pn = 0.0;
        for (int j = 0; j < m; ++j) {
            pn = fma(coef[j], coef[j], pn);
        }
        scal[0] = pn;
        scal[1] = sum_parts(part + (m & 1) * nb, nb);
    }
}

__global__ void __launch_bounds__(AP_THREADS)
    k_append_store(double w, double *__restrict__ v, float *__restrict__ Bo, size_t ldbo,
                   float *__restrict__ BoC, int n, int m, const float *__restrict__ y,
                   double *__restrict__ part)
{
    __shared__ double red[32];
    int lo, hi;
    block_rows(n, gridDim.x, blockIdx.x, lo, hi);
    double acc = 0.0;
    for (int i = lo + threadIdx.x; i < hi; i += AP_THREADS) {
        const double vi = v[i] / w;
        v[i] = vi;
        const float vf = (float)vi;
        Bo[(size_t)i * ldbo + m] = vf;
        BoC[(size_t)m * n + i] = vf;
        acc = fma((double)vf, (double)y[i], acc);
    }
    const double bs = block_sum<AP_THREADS>(acc, red);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = bs;
    }
}

__global__ void k_sum_into(const double *__restrict__ part, int nb, double *__restrict__ out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *out = sum_parts(part, nb);
    }
}

constexpr int CS_THREADS = 256;
__global__ void __launch_bounds__(CS_THREADS)
    k_colsumsq(const float *__restrict__ X, size_t ldX, int n, int p, double *__restrict__ part)
{
    __shared__ double red[32];
    const int j = blockIdx.y;
    int lo, hi;
    block_rows(n, gridDim.x, blockIdx.x, lo, hi);
    double acc = 0.0;
    for (int i = lo + threadIdx.x; i < hi; i += CS_THREADS) {
        const double x = (double)X[(size_t)i + (size_t)j * ldX];
        acc = fma(x, x, acc);
    }
    const double bs = block_sum<CS_THREADS>(acc, red);
    if (threadIdx.x == 0) {
        part[(size_t)blockIdx.x * p + j] = bs;
    }
}

int tgemm_splits(int n, int col_tiles, int comp_tiles, int *rows_per_split)
{
    const int target = 152 * 4;
    int splits = (int)ceil_div((size_t)target, (size_t)col_tiles * comp_tiles);
    const int max_splits = (int)ceil_div((size_t)n, 256);
    splits = std::max(1, std::min(splits, max_splits));
    *rows_per_split = (int)round_up(ceil_div((size_t)n, (size_t)splits), TG_ROWS);
    splits = (int)ceil_div((size_t)n, (size_t)*rows_per_split);
    return std::max(splits, 1);
}

}  // namespace

int append_blocks(int n) { return (int)std::max<size_t>(1, std::min<size_t>(608, ceil_div(n, 2048))); }

// Largest split-K workspace any column count in [1, P] needs (fewer columns
// mean more splits, so the maximum is not always at P itself).
size_t project_tpart_elems(int n, int m, int P)
{
    size_t best = 0;
    const int comp_tiles = (int)ceil_div(std::max(m, 1), TG_COMPS);
    for (int ct = 1; ct <= (int)ceil_div(std::max(P, 1), TG_COLS); ++ct) {
        const int cols = std::min(ct * TG_COLS, std::max(P, 1));
        int rps;
        const int splits = tgemm_splits(n, ct, comp_tiles, &rps);
        best = std::max(best, (size_t)splits * cols * std::max(m, 1));
    }
    return best;
}

size_t project_part_elems(int n, int P) { return ceil_div(n, PJ_THREADS) * (size_t)P; }

template <class Src>
void tgemm_fp64(cudaStream_t st, const Src &src, const float *Bo, size_t ldbo, int n, int m,
                int P, double *T, double *Tpart, size_t tpart_elems, long long *launches)
{
    if (P <= 0 || m <= 0) {
        return;
    }
    int rps;
    const int col_tiles = (int)ceil_div(P, TG_COLS), comp_tiles = (int)ceil_div(m, TG_COMPS);
    const int splits = tgemm_splits(n, col_tiles, comp_tiles, &rps);
    verify((size_t)splits * P * m <= tpart_elems, "internal: T workspace too small", 2);
    k_tgemm<Src><<<dim3(col_tiles, splits, comp_tiles), TG_THREADS, 0, st>>>(src, Bo, ldbo, n, m,
                                                                           P, rps, Tpart);
    LAUNCH_CHECK();
    const size_t cnt = (size_t)P * m;
    k_reduce_splits<<<(unsigned)ceil_div(cnt, 256), 256, 0, st>>>(Tpart, splits, cnt, T);
    LAUNCH_CHECK();
    *launches += 2;
}

template void tgemm_fp64<FillSrc>(cudaStream_t, const FillSrc &, const float *, size_t, int, int,
                                  int, double *, double *, size_t, long long *);
template void tgemm_fp64<StoredSrc>(cudaStream_t, const StoredSrc &, const float *, size_t, int,
                                    int, int, double *, double *, size_t, long long *);

template <class Src>
void project_fp64(cudaStream_t st, const Src &src, const float *Bo, size_t ldbo, int n, int m,
                  int P, const int *out_col, float *Bx, size_t ldBx, double *s_out,
                  const ProjectScratch &ws, long long *launches)
{
    if (P <= 0) {
        return;
    }
    tgemm_fp64(st, src, Bo, ldbo, n, m, P, ws.T, ws.Tpart, ws.tpart_elems, launches);
    const int rb = (int)ceil_div(n, PJ_THREADS);
    verify((size_t)rb * P <= ws.part_elems, "internal: partial workspace too small", 2);
    const size_t smem = sizeof(double) * PJ_COLS * std::max(m, 1);
    if (smem > 48 * 1024) {
        CUDA_CHECK(cudaFuncSetAttribute(k_project<Src>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
    }
    k_project<Src><<<dim3(rb, (unsigned)ceil_div(P, PJ_COLS)), PJ_THREADS, smem, st>>>(
        src, Bo, ldbo, n, m, P, ws.T, out_col, Bx, ldBx, ws.part);
    LAUNCH_CHECK();
    k_reduce_cols<<<(unsigned)ceil_div(P, 128), 128, 0, st>>>(ws.part, rb, P, s_out);
    LAUNCH_CHECK();
    *launches += 2;
}

template void project_fp64<FillSrc>(cudaStream_t, const FillSrc &, const float *, size_t, int,
                                    int, int, const int *, float *, size_t, double *,
                                    const ProjectScratch &, long long *);
template void project_fp64<StoredSrc>(cudaStream_t, const StoredSrc &, const float *, size_t,
                                      int, int, int, const int *, float *, size_t, double *,
                                      const ProjectScratch &, long long *);

void dgks_gate(cudaStream_t st, const double *T, int m, int P, const double *s, double tol,
               int *fired, int *nfired, long long *launches)
{
    CUDA_CHECK(cudaMemsetAsync(nfired, 0, sizeof(int), st));
    k_gate<<<(unsigned)ceil_div(P, 128), 128, 0, st>>>(T, m, P, s, tol, fired, nfired);
    LAUNCH_CHECK();
    *launches += 1;
}

void scatter_s(cudaStream_t st, const int *fired, int nf, const double *snew, double *s,
               long long *launches)
{
    k_scatter_s<<<(unsigned)ceil_div(nf, 128), 128, 0, st>>>(fired, nf, snew, s);
    LAUNCH_CHECK();
    *launches += 1;
}

void normalize_ybx(cudaStream_t st, float *Bx, size_t ldBx, int n, int P, const double *s,
                   double tol, const float *y, bool store, double *ybx, double *part,
                   long long *launches)
{
    const int rb = (int)ceil_div(n, NM_THREADS);
    k_normalize<<<dim3(rb, (unsigned)ceil_div(P, NM_COLS)), NM_THREADS, 0, st>>>(
        Bx, ldBx, n, P, s, tol, y, store, part);
    LAUNCH_CHECK();
    k_reduce_cols<<<(unsigned)ceil_div(P, 128), 128, 0, st>>>(part, rb, P, ybx);
    LAUNCH_CHECK();
    *launches += 2;
}

size_t normalize_part_elems(int n, int P) { return ceil_div(n, NM_THREADS) * (size_t)P; }

void sweep_fp64(cudaStream_t st, const SweepTask *tasks, int ntasks, const int *perm,
                const float *xsort, const float *y, const float *B, size_t ldB,
                const int *cand_b, const float *Bx, size_t ldBx, const float *Bo, size_t ldbo,
                const double *ybo, const double *ybx, int n, int m, int head, int tail,
                int min_span, double tol, double *hsse, int *hrow, long long *launches)
{
    if (ntasks <= 0) {
        return;
    }
    const size_t smem = sizeof(float) * SW_ROWS * (size_t)(m | 1);
    const int comps = m + 1;
#define LAUNCH_SWEEP(CPL)                                                                      \
    do {                                                                                       \
        if (smem > 48 * 1024) {                                                                \
            CUDA_CHECK(cudaFuncSetAttribute(k_sweep<CPL>,                                      \
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                                            (int)smem));                                       \
        }                                                                                      \
        k_sweep<CPL><<<ntasks, SW_THREADS, smem, st>>>(tasks, perm, xsort, y, B, ldB, cand_b,  \
                                                       Bx, ldBx, Bo, ldbo, ybo, ybx, n, m,     \
                                                       head, tail, min_span, tol, hsse, hrow); \
    } while (0)
    if (comps <= 32) {
        LAUNCH_SWEEP(1);
    } else if (comps <= 64) {
        LAUNCH_SWEEP(2);
    } else if (comps <= 128) {
        LAUNCH_SWEEP(4);
    } else if (comps <= 256) {
        LAUNCH_SWEEP(8);
    } else if (comps <= 512) {
        LAUNCH_SWEEP(16);
    } else {
        throw Error(1, "the GPU hinge sweep supports at most 511 basis functions");
    }
#undef LAUNCH_SWEEP
    LAUNCH_CHECK();
    *launches += 1;
}

void sort_columns(cudaStream_t st, const float *X, size_t ldX, const float *s, int n,
                  const int *cols, int ncols, int *perm, float *xsort, DevBuf &keys,
                  DevBuf &vals, DevBuf &tmp, long long *launches)
{
    keys.ensure(2 * sizeof(float) * (size_t)n);
    vals.ensure(sizeof(int) * (size_t)n);
    size_t need = 0;
    float *k_in = keys.as<float>(), *k_out = keys.as<float>() + n;
    CUDA_CHECK(cub::DeviceRadixSort::SortPairsDescending(nullptr, need, k_in, k_out,
                                                         vals.as<int>(), perm, n, 0, 32, st));
    tmp.ensure(std::max<size_t>(need, 16));
    const unsigned nb = (unsigned)ceil_div(n, 256);
    for (int q = 0; q < ncols; ++q) {
        const int c = cols[q];
        int *pc = perm + (size_t)c * n;
        k_sort_keys<<<nb, 256, 0, st>>>(X, ldX, n, c, k_in, vals.as<int>());
        LAUNCH_CHECK();
        size_t bytes = tmp.bytes;
        CUDA_CHECK(cub::DeviceRadixSort::SortPairsDescending(tmp.ptr, bytes, k_in, k_out,
                                                             vals.as<int>(), pc, n, 0, 32, st));
        k_gather_scaled<<<nb, 256, 0, st>>>(X, ldX, s, n, c, pc, xsort + (size_t)c * n);
        LAUNCH_CHECK();
        *launches += 2 + 4;  // our two kernels plus the radix-sort passes
    }
}

void fill_outputs(cudaStream_t st, int rows, int m, double *lin, double *hin, double *cut,
                  long long *launches)
{
    const size_t cnt = (size_t)rows * m;
    if (cnt == 0) {
        return;
    }
    k_fill_outputs<<<(unsigned)ceil_div(cnt, 256), 256, 0, st>>>(cnt, lin, hin, cut);
    LAUNCH_CHECK();
    *launches += 1;
}

void assemble_outputs(cudaStream_t st, int P, const int *cand_x, const int *cand_b, int m,
                      const double *ybx, const double *hsse, const int *hrow, const float *X,
                      size_t ldX, bool linear_only, double *lin, double *hin, double *cut,
                      long long *launches)
{
    if (P <= 0) {
        return;
    }
    k_assemble<<<(unsigned)ceil_div(P, 128), 128, 0, st>>>(P, cand_x, cand_b, m, ybx, hsse, hrow,
                                                         X, ldX, linear_only, lin, hin, cut);
    LAUNCH_CHECK();
    *launches += 1;
}

void append_fill(cudaStream_t st, char type, const float *X, size_t ldX, const float *s,
                 int xcol, float *B, size_t ldB, int bcol, int m, float h, int n,
                 const AppendScratch &ws, long long *launches)
{
    k_append_fill<<<ws.nblocks, AP_THREADS, 0, st>>>(type, X, ldX, s, xcol, B, ldB, bcol, m, h, n,
                                                     ws.v, ws.part);
    LAUNCH_CHECK();
    k_append_scale<<<ws.nblocks, AP_THREADS, 0, st>>>(B, ldB, m, n, ws.part, ws.nblocks);
    LAUNCH_CHECK();
    *launches += 2;
}

void mgs_pass(cudaStream_t st, const float *BoC, int n, int m, const AppendScratch &ws,
              long long *launches)
{
    for (int j = 0; j <= m; ++j) {
        k_mgs_step<<<ws.nblocks, AP_THREADS, 0, st>>>(BoC, n, m, j, ws.v, ws.part, ws.nblocks,
                                                      ws.coef);
        LAUNCH_CHECK();
    }
    k_mgs_finish<<<1, 32, 0, st>>>(ws.part, ws.nblocks, m, ws.coef, ws.scal);
    LAUNCH_CHECK();
    *launches += m + 2;
}

void append_store(cudaStream_t st, double w, float *Bo, size_t ldbo, float *BoC, int n, int m,
                  const float *y, const AppendScratch &ws, long long *launches)
{
    k_append_store<<<ws.nblocks, AP_THREADS, 0, st>>>(w, ws.v, Bo, ldbo, BoC, n, m, y, ws.part);
    LAUNCH_CHECK();
    k_sum_into<<<1, 32, 0, st>>>(ws.part, ws.nblocks, ws.scal + 2);
    LAUNCH_CHECK();
    *launches += 2;
}

void column_sumsq(cudaStream_t st, const float *X, size_t ldX, int n, int p, double *out,
                  double *part, long long *launches)
{
    const int nb = append_blocks(n);
    verify(p <= 65535, "more than 65535 X columns");
    k_colsumsq<<<dim3(nb, p), CS_THREADS, 0, st>>>(X, ldX, n, p, part);
    LAUNCH_CHECK();
    k_reduce_cols<<<(unsigned)ceil_div(p, 128), 128, 0, st>>>(part, nb, p, out);
    LAUNCH_CHECK();
    *launches += 2;
}

}  // namespace mgpu
