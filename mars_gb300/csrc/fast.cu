// Fast (ranking) pass of the mixed-precision forward pass.
//
// Projection: FP32 split-K GEMMs (T = Bo^T v, then v - Bo T), applied twice
// so the second pass re-orthogonalises the first one's residual (the role of
// the reference's DGKS step, kernels.cc:384-395), then FP32 norms with FP64
// block sums.
//
// Hinge sweep: the reference's recurrences (marsalgo.cc:576-649 with
// covariates_impl :91-151) in chunks of sorted rows: inside a chunk the
// increments are f32 (the running sums of products exact as f32 pairs),
// across chunks the running values are carried as float-float pairs:
//   g_c(i) = G_c + q_c(i)
//   f_c(i) = F_c + G_c D(i) + e_c(i)      (D(i): sum of the chunk's deltas to row i)
// with e_c += d q_c, q_c += b x_c. Besides the basis columns and the
// candidate column, two more components carry the scalar recurrences: x = y
// (g = vb, f = w) and x = b (g = b2, f = bd), and K = k0 + k1 follows as
//   K(i) = K + 2 F_b D(i) + G_b D(i)^2 + kl(i),   kl += d^2 q_b + 2 d e_b.
// A grid row stores only the f32 increments; the scores are rebuilt from the
// chunk's float-float anchors, 32 grid rows at a time (lane = grid row).
#include "fast.cuh"

#include <algorithm>
#include <cstdlib>

namespace mgpu {
namespace {

__device__ __forceinline__ float fast_scale(double s, double tol)
{
    return s > tol ? (float)(1.0 / sqrt(s + tol)) : 0.0f;
}

// ---------------------------------------------------------------------------
// Split-K T = Bo^T v: block = 32 candidates x 32 components over one row range;
// thread = one component x 4 candidates.
// ---------------------------------------------------------------------------
constexpr int FT_ROWS = 32, FT_THREADS = 256;

template <class Src>
__global__ void __launch_bounds__(FT_THREADS)
    k_fast_tgemm(Src src, const float *__restrict__ BoC, int n, int m, int P, int rps,
                 float *__restrict__ Tp)
{
    __shared__ float sA[FT_ROWS][33];
    __shared__ float sV[FT_ROWS][33];
    const int t = threadIdx.x, kk = t & 31, jq = t >> 5;
    const int j0 = blockIdx.x * 32, k0 = blockIdx.y * 32, split = blockIdx.z;
    const int r0 = split * rps, r1 = min(n, r0 + rps);
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int rb = r0; rb < r1; rb += FT_ROWS) {
        for (int e = t; e < FT_ROWS * 32; e += FT_THREADS) {
            const int rr = e & 31, cc = e >> 5, i = rb + rr;
            sA[rr][cc] = (i < r1 && k0 + cc < m) ? BoC[i + (size_t)(k0 + cc) * n] : 0.f;
            sV[rr][cc] = (i < r1 && j0 + cc < P) ? src((size_t)i, j0 + cc) : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int rr = 0; rr < FT_ROWS; ++rr) {
            const float a = sA[rr][kk];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                acc[q] = fmaf(a, sV[rr][jq * 4 + q], acc[q]);
            }
        }
        __syncthreads();
    }
    if (k0 + kk < m) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int j = j0 + jq * 4 + q;
            if (j < P) {
                Tp[((size_t)split * P + j) * m + k0 + kk] = acc[q];
            }
        }
    }
}

__global__ void k_fast_treduce(const float *__restrict__ Tp, int ks, size_t count,
                               float *__restrict__ T)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) {
        double a = 0.0;
        for (int q = 0; q < ks; ++q) {
            a += (double)Tp[(size_t)q * count + e];
        }
        T[e] = (float)a;
    }
}

// Bx[i, j] = v(i, j) - sum_k Bo[i, k] T[j][k]; block = 64 rows x 64 candidates,
// thread = one row x 16 candidates.
constexpr int FP_ROWS = 64, FP_COLS = 64, FP_THREADS = 256, FP_PER = 16;

template <class Src>
__global__ void __launch_bounds__(FP_THREADS)
    k_fast_project(Src src, const float *__restrict__ BoC, int n, int m, int P,
                   const float *__restrict__ T, float *__restrict__ Bx)
{
    extern __shared__ float sT[];  // [FP_COLS][m]
    const int t = threadIdx.x, ri = t % FP_ROWS, cg = t / FP_ROWS;
    const int j0 = blockIdx.y * FP_COLS;
    for (int e = t; e < FP_COLS * m; e += FP_THREADS) {
        const int q = e / m, k = e % m, j = j0 + q;
        sT[e] = j < P ? T[(size_t)j * m + k] : 0.f;
    }
    __syncthreads();
    const int i = blockIdx.x * FP_ROWS + ri;
    if (i >= n) {
        return;
    }
    float acc[FP_PER];
#pragma unroll
    for (int q = 0; q < FP_PER; ++q) {
        acc[q] = 0.f;
    }
    for (int k = 0; k < m; ++k) {
        const float a = BoC[i + (size_t)k * n];
#pragma unroll
        for (int q = 0; q < FP_PER; ++q) {
            acc[q] = fmaf(a, sT[(cg * FP_PER + q) * m + k], acc[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < FP_PER; ++q) {
        const int j = j0 + cg * FP_PER + q;
        if (j < P) {
            const float v = src((size_t)i, j);
            Bx[i + (size_t)j * n] = v - acc[q];
        }
    }
}

// s[j] = ||Bx_j||^2, ybx[j] = scale(s_j) * (Bx_j . y): FP32 per thread, FP64 across.
__global__ void __launch_bounds__(256)
    k_fast_norms(const float *__restrict__ Bx, int n, const float *__restrict__ y, double tol,
                 double *__restrict__ s, double *__restrict__ ybx)
{
    __shared__ double red[2][8];
    const int j = blockIdx.x, t = threadIdx.x;
    const float *col = Bx + (size_t)j * n;
    float a = 0.f, b = 0.f;
    for (int i = t; i < n; i += 256) {
        const float v = col[i];
        a = fmaf(v, v, a);
        b = fmaf(v, y[i], b);
    }
    double da = warp_sum((double)a), db = warp_sum((double)b);
    if ((t & 31) == 0) {
        red[0][t >> 5] = da;
        red[1][t >> 5] = db;
    }
    __syncthreads();
    if (t == 0) {
        double sa = 0.0, sb = 0.0;
        for (int w = 0; w < 8; ++w) {
            sa += red[0][w];
            sb += red[1][w];
        }
        s[j] = sa;
        ybx[j] = (double)fast_scale(sa, tol) * sb;
    }
}

// Per candidate j (parent b = B[:, cand_b[j]], input x = X[:, cand_x[j]] * s):
// mom[3 j + k] = sum_i b_i^2 x_i^k, k = 0, 1, 2 (sum b^2 x^2 is also the raw
// squared norm of the candidate column x b). They only set flag thresholds, so
// FP32 per thread and FP64 across threads (an FP64 sum per row would make the
// kernel FP64-pipe bound).
__global__ void __launch_bounds__(256) k_parent_moments(FillSrc src, int n, double *__restrict__ mom)
{
    __shared__ double red[3][8];
    const int j = blockIdx.x, t = threadIdx.x;
    const int xc = src.cand_x[j];
    const float *bcol = src.B + (size_t)src.cand_b[j] * src.ldB;
    const float *xcol = src.X + (size_t)xc * src.ldX;
    const float sx = src.s[xc];
    float f0 = 0.f, f1 = 0.f, f2 = 0.f;
    for (int i = t; i < n; i += 256) {
        const float b = bcol[i], x = xcol[i] * sx;
        const float b2 = b * b, b2x = b2 * x;
        f0 += b2;
        f1 += b2x;
        f2 = fmaf(b2x, x, f2);
    }
    double a0 = warp_sum((double)f0), a1 = warp_sum((double)f1), a2 = warp_sum((double)f2);
    if ((t & 31) == 0) {
        red[0][t >> 5] = a0;
        red[1][t >> 5] = a1;
        red[2][t >> 5] = a2;
    }
    __syncthreads();
    if (t < 3) {
        double v = 0.0;
        for (int w = 0; w < 8; ++w) {
            v += red[t][w];
        }
        mom[3 * (size_t)j + t] = v;
    }
}

// s and ybx of row-major candidate columns, in two deterministic steps: block
// (32 candidates, one chunk of FN_ROWS rows): lane = candidate, warp w takes
// rows w, w + 8, ... of the chunk, FP32 per thread, FP64 across the warps in
// a fixed order, into part[chunk][j][2]; then k_fast_norms_rows_done adds the
// chunks in order.
constexpr int FN_ROWS = 4096;

__global__ void __launch_bounds__(256)
    k_fast_norms_rows(const float *__restrict__ Bx, size_t ldr, int n, const float *__restrict__ y,
                      int P, double *__restrict__ part)
{
    __shared__ double red[2][8][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + lane, ch = blockIdx.y;
    const int r0 = ch * FN_ROWS, r1 = min(n, r0 + FN_ROWS);
    float a = 0.f, b = 0.f;
    if (j < P) {
#pragma unroll 4
        for (int i = r0 + w; i < r1; i += 8) {
            const float v = Bx[(size_t)i * ldr + j];
            a = fmaf(v, v, a);
            b = fmaf(v, y[i], b);
        }
    }
    red[0][w][lane] = (double)a;
    red[1][w][lane] = (double)b;
    __syncthreads();
    if (w < 2 && j < P) {
        double t = 0.0;
        for (int q = 0; q < 8; ++q) {
            t += red[w][q][lane];
        }
        part[((size_t)ch * P + j) * 2 + w] = t;
    }
}

__global__ void k_fast_norms_rows_done(const double *__restrict__ part, int nch, int P,
                                       double tol, double *__restrict__ s, double *__restrict__ ybx)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < P) {
        double a = 0.0, b = 0.0;
        for (int c = 0; c < nch; ++c) {
            a += part[((size_t)c * P + j) * 2];
            b += part[((size_t)c * P + j) * 2 + 1];
        }
        s[j] = a;
        ybx[j] = (double)fast_scale(a, tol) * b;
    }
}

// Column-major (ld n) candidate columns to the row-major layout (ld ldr).
__global__ void k_fast_to_rows(const float *__restrict__ Bc, int n, int P, float *__restrict__ Br,
                               size_t ldr)
{
    __shared__ float t[32][33];
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int i = i0 + threadIdx.x, j = j0 + q;
        t[q][threadIdx.x] = (i < n && j < P) ? Bc[(size_t)j * n + i] : 0.f;
    }
    __syncthreads();
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int i = i0 + q, j = j0 + threadIdx.x;
        if (i < n && j < P) {
            Br[(size_t)i * ldr + j] = t[threadIdx.x][q];
        }
    }
}

// ---------------------------------------------------------------------------
// Chunked sweep. Block = one input column, one direction and up to W
// candidates (warps 0..W-1, lane = component) plus two loader warps that stage
// each 32-row stage with cp.async: warp W the gathered f32 Bo rows (16 bytes
// per lane), warp W+1, lanes over rows, the sorted parent and candidate
// values, y and x, then the f32 deltas (copies in flight are limited per
// warp, so the staging is split).
//
// Directions. Forward tasks sweep the descending order from the top and score
// the cuts of its first half. Near the bottom the hinge (x - t)+ b differs
// from (x - t) b -- which lies in the span of the parent and the candidate --
// only on the few rows below the cut, so den = K - ff cancels to ~1e-11 K and
// f32 increments cannot resolve it; but the mirror hinge (t - x)+ b has the
// same residual, and the mirror tasks sweep from the bottom (the same
// recurrences on the reversed order, deltas x_cur - x_prev) and score the
// cuts of the second half, where that mirror is small.
//
// Arithmetic (no FP64 instruction: the FP64 pipe of this GPU issues one warp
// instruction per 64 cycles per sub-partition). A chunk is FS_CHUNK stages
// (64 rows). Inside a chunk, per component, e += d q in f32 and q += b x with
// the f32 products summed exactly as an unevaluated pair (q_hi, q_lo) by
// Knuth's two-sum: the rounding of a long f32 running sum, not of its
// products, is what would otherwise dominate the error of den (measured on a
// fit of n = 1e5: ~20x the error of the exact sum). At a chunk end
// the carries (float-float pairs, Dekker's arithmetic) take the increments,
//   K += Dc (2 F_b + G_b Dc) + kl,   F += G Dc + e,   G += q,
// with Dc = x_base - x_end formed exactly. Scoring, 32 grid rows at a time:
// per chunk, the float-float sums over the basis and candidate components
//   FF = sum F_c^2, FG = sum F_c G_c, GG = sum G_c^2, Fy = sum F_c yc_c, Gy = sum G_c yc_c
// (lane = chunk and sum) give the chunk's anchors, in which the large terms
// cancel in float-float and only the differences are rounded to f32:
//   A0 = K - FF, A1 = 2 (F_b - FG), A2 = G_b - GG, B0 = Fy - F_y, B1 = Gy - G_y;
// then per grid row (lane = grid row), in f32, with D = x_base - x exact as a pair,
//   den = A0 + D (A1 + D A2) + kl - 2 (Fe + D Ge) - ee,   uw = B0 + D B1 + ey - e_y,
// Fe = sum F_c e_c, Ge = sum G_c e_c, ee = sum e_c^2, ey = sum yc_c e_c.
// ---------------------------------------------------------------------------
constexpr int FS_ROWS = 32, FS_CHUNK = 2, FS_SNAP = 32, FS_HIST = 4, FS_NSUM = 5, FS_MAXW = 8;
constexpr int FS_RS = FS_ROWS + 1;  // stride of the staged per-row arrays: each in its own banks

using FastTask = FastTaskRec;  // dir 0: forward (first half of the cuts), 1: mirror (second half)

// Error-free transformations (Knuth's two-sum, Dekker's fast two-sum and
// product with a fused multiply-add); the explicit _rn intrinsics keep the
// compiler from contracting or reassociating them.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &err)
{
    s = __fadd_rn(a, b);
    const float bv = __fsub_rn(s, a);
    const float av = __fsub_rn(s, bv);
    err = __fadd_rn(__fsub_rn(a, av), __fsub_rn(b, bv));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &err)
{
    s = __fadd_rn(a, b);
    err = __fsub_rn(b, __fsub_rn(s, a));
}

// (ah, al) += (bh, bl)
__device__ __forceinline__ void ff_add(float &ah, float &al, float bh, float bl)
{
    float s, e;
    two_sum(ah, bh, s, e);
    e = __fadd_rn(e, __fadd_rn(al, bl));
    fast_two_sum(s, e, ah, al);
}

// (ph, pl) = (ah, al) (bh, bl)
__device__ __forceinline__ void ff_mul(float ah, float al, float bh, float bl, float &ph,
                                       float &pl)
{
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    fast_two_sum(p, e, ph, pl);
}

// (ah - bh) + (al - bl) rounded to f32
__device__ __forceinline__ float ff_diff(float ah, float al, float bh, float bl)
{
    float s, e;
    two_sum(ah, -bh, s, e);
    return __fadd_rn(s, __fadd_rn(e, __fsub_rn(al, bl)));
}

struct FastSweepSmem {
    size_t hFh, hFl, hGh, hGl, hK, hXb, cA, csum, sE, sKL, sCh, srow, sXv, ycf, bo, raw, dsm,
        zero, total;
    __host__ __device__ FastSweepSmem(int m, int W, int S)
    {
        const size_t ncs = (size_t)((m + 3) | 1);  // odd stride: conflict-free column reads
        size_t o = 0;
        hFh = o;  // [W][FS_HIST][ncs] carries at chunk starts, float-float
        o += 4 * (size_t)W * FS_HIST * ncs;
        hFl = o;
        o += 4 * (size_t)W * FS_HIST * ncs;
        hGh = o;
        o += 4 * (size_t)W * FS_HIST * ncs;
        hGl = o;
        o += 4 * (size_t)W * FS_HIST * ncs;
        hK = o;  // [W][FS_HIST][2]
        o += 4 * (size_t)W * FS_HIST * 2;
        hXb = o;  // [FS_HIST] x at the chunk's base
        o += 4 * FS_HIST;
        cA = o;  // [W][FS_HIST][FS_NSUM] f32 anchors A0, A1, A2, B0, B1
        o += 4 * (size_t)W * FS_HIST * FS_NSUM;
        csum = o;  // [W][FS_HIST][FS_NSUM][2] float-float chunk sums
        o += 4 * (size_t)W * FS_HIST * FS_NSUM * 2;
        sE = o;  // [W][FS_SNAP][ncs] f32 increments e at grid rows
        o += 4 * (size_t)W * FS_SNAP * ncs;
        sKL = o;  // [W][FS_SNAP]
        o += 4 * (size_t)W * FS_SNAP;
        sCh = o;  // [FS_SNAP] chunk history index of the grid row
        o += 4 * FS_SNAP;
        srow = o;  // [FS_SNAP] sorted row of the grid row
        o += 4 * FS_SNAP;
        sXv = o;  // [FS_SNAP] f32 x (the knot) of the grid row
        o += 4 * FS_SNAP;
        ycf = o;  // [W][m + 1][2] float-float y coefficients (ybo, then ybx)
        o += 8 * (size_t)W * (m + 1);
        o = (o + 15) / 16 * 16;  // 16-byte cp.async destinations
        bo = o;  // [S][FS_ROWS][mp] f32, row stride mp = m rounded up to 4
        o += 4 * (size_t)S * FS_ROWS * ((m + 3) / 4 * 4);
        raw = o;  // [S][(2W + 1) * FS_RS + FS_ROWS + 1] f32: B, Bx per candidate, y, x
        o += 4 * (size_t)S * ((2 * W + 1) * FS_RS + FS_ROWS + 1);
        dsm = o;  // [2][FS_ROWS] f32 deltas
        o += 4 * 2 * FS_ROWS;
        zero = o;  // one f32 zero
        o += 4;
        total = (o + 15) / 16 * 16;
    }
};

// RB: blocks of the largest size meant to reside per SM (the register cap
// follows from it).
template <int CPL, int S, int RB>
__global__ void __launch_bounds__(32 * (FS_MAXW + 2), RB)
    k_fast_sweep(const FastTask *__restrict__ tasks, const int *__restrict__ perm,
                 const float *__restrict__ xsort, const float *__restrict__ ysort,
                 const FastSweepCols cols,
                 const float *__restrict__ BoR, size_t ldbo, const double *__restrict__ ybo,
                 const double *__restrict__ ybx, const double *__restrict__ mom, int n, int m,
                 int head, int tail, int mid, int min_span, double tol, double cut_rel,
                 double *__restrict__ hsse, int *__restrict__ hrow, int *__restrict__ hflag)
{
    extern __shared__ __align__(16) unsigned char sm[];
    const int W = (blockDim.x >> 5) - 2;  // candidate warps; then the two loaders
    const int NC = m + 3;  // basis columns, candidate, y, b
    const int NCS = NC | 1;
    const int U = (m + 3) / 4, MP = 4 * U;  // 16-byte units per Bo row, padded row stride
    const int RAW = (2 * W + 1) * FS_RS + FS_ROWS + 1;
    const FastSweepSmem L(m, W, S);
    float *hFh = reinterpret_cast<float *>(sm + L.hFh);
    float *hFl = reinterpret_cast<float *>(sm + L.hFl);
    float *hGh = reinterpret_cast<float *>(sm + L.hGh);
    float *hGl = reinterpret_cast<float *>(sm + L.hGl);
    float *hK = reinterpret_cast<float *>(sm + L.hK);
    float *hXb = reinterpret_cast<float *>(sm + L.hXb);
    float *cA = reinterpret_cast<float *>(sm + L.cA);
    float *csum = reinterpret_cast<float *>(sm + L.csum);
    float *sE = reinterpret_cast<float *>(sm + L.sE);
    float *sKL = reinterpret_cast<float *>(sm + L.sKL);
    int *sCh = reinterpret_cast<int *>(sm + L.sCh);
    int *srow = reinterpret_cast<int *>(sm + L.srow);
    float *sXv = reinterpret_cast<float *>(sm + L.sXv);
    float *sycf = reinterpret_cast<float *>(sm + L.ycf);
    float *sbo = reinterpret_cast<float *>(sm + L.bo);
    float *sraw4 = reinterpret_cast<float *>(sm + L.raw);
    float *dsm = reinterpret_cast<float *>(sm + L.dsm);
    float *zero = reinterpret_cast<float *>(sm + L.zero);
    if (threadIdx.x == 0) {
        *zero = 0.f;
    }

    const FastTask task = tasks[blockIdx.x];
    const bool rev = task.dir != 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool cwarp = warp < task.count;
    const bool lwarp = warp == W;      // loader of the Bo rows
    const bool rwarp = warp == W + 1;  // loader of the per-candidate arrays, y, x
    const int *pk = perm + (size_t)task.xcol * n;
    const float *xs = xsort + (size_t)task.xcol * n;
    const float *ys = ysort + (size_t)task.xcol * n;
    // loader of the per-candidate arrays: lane q holds candidate q's parent
    // column and normalisation
    const int pcol = rwarp && lane < task.count ? cols.cand_b[task.cand0 + lane] : 0;
    const float pscale =
        rwarp && lane < task.count ? fast_scale(cols.s[task.cand0 + lane], tol) : 0.0f;
    for (int e = threadIdx.x; e < W * (m + 1); e += blockDim.x) {
        const int w = e / (m + 1), c = e % (m + 1);
        const double v = c < m ? ybo[c] : (w < task.count ? ybx[task.cand0 + w] : 0.0);
        const float hi = (float)v;
        sycf[2 * e] = hi;
        sycf[2 * e + 1] = (float)(v - (double)hi);
    }
    __syncthreads();

    // Processing step s visits sorted row idx(s); the task's cuts are the grid
    // rows g = head + 1 + k min_span <= tail - 1 on its side of mid.
    const int len = rev ? n - 1 - mid : mid + 1;
    auto idx = [&](int s) { return rev ? n - 1 - s : s; };
    const long g_last = tail - 1 >= head + 1
                            ? (long)head + 1 + (long)((tail - 1 - (head + 1)) / min_span) * min_span
                            : -1;
    int next_grid, last_step;  // in processing steps
    if (!rev) {
        next_grid = head + 1;
        last_step = g_last < 0 ? -1 : (int)(g_last < (long)mid ? g_last : (long)mid);
    } else {
        next_grid = g_last < 0 ? len : (int)((long)n - 1 - g_last);  // largest grid row first
        last_step = g_last < 0 ? -1 : n - 1 - (mid + 1);
    }
    const int nstages = (len + FS_ROWS - 1) / FS_ROWS;

    int pf_k = 0;
    auto prefetch = [&](int sq) {
        const int s = sq * FS_ROWS + lane;
        if (sq < nstages && s < len) {
            pf_k = pk[idx(s)];
        }
    };
    auto issue_bo = [&](int sq) {
        const int sg = sq % S, s0 = sq * FS_ROWS;
        const int rows = min(FS_ROWS, len - s0);
        const int k = pf_k;
        float *bo = sbo + (size_t)sg * FS_ROWS * MP;
        for (int e0 = 0; e0 < FS_ROWS * U; e0 += 32) {
            const int e = e0 + lane, r = e / U, u = e - r * U;
            const int kr = __shfl_sync(0xffffffffu, k, r < FS_ROWS ? r : 0);
            if (r < rows) {
                cp_async<16>(bo + r * MP + 4 * u, BoR + (size_t)kr * ldbo + 4 * u);
            }
        }
    };
    auto issue_raw = [&](int sq) {
        const int sg = sq % S, s0 = sq * FS_ROWS;
        const int rows = min(FS_ROWS, len - s0);
        float *rw = sraw4 + (size_t)sg * RAW;
        const bool ok = lane < rows;
        const int i = ok ? idx(s0 + lane) : 0;
        const int pi = ok ? pk[i] : 0;  // the row of sorted position i
        for (int cw = 0; cw < task.count; ++cw) {
            const int bc = __shfl_sync(0xffffffffu, pcol, cw);
            cp_async4(rw + cw * FS_RS + lane, cols.BR + (size_t)pi * cols.ldBR + bc, ok);
            cp_async4(rw + (W + cw) * FS_RS + lane,
                      cols.Bx + (size_t)pi * cols.ldr + task.cand0 + cw, ok);
        }
        cp_async4(rw + 2 * W * FS_RS + lane, ys + i, ok);
        cp_async4(rw + (2 * W + 1) * FS_RS + 1 + lane, xs + i, ok);
        if (lane == 0) {
            cp_async4(rw + (2 * W + 1) * FS_RS, xs + (s0 > 0 ? idx(s0 - 1) : 0), s0 > 0);
        }
    };
    // Stage sq (landed): the f32 deltas of its rows (lanes = rows), formed as
    // the reference forms them (marsalgo.cc:523-525).
    // and the candidate columns normalised in place, f32(Bx * scale).
    auto deltas = [&](int sq) {
        float *rwl = sraw4 + (size_t)(sq % S) * RAW;
        const float *xr = rwl + (2 * W + 1) * FS_RS;
        const int h = sq & 1, s = sq * FS_ROWS + lane;
        const bool ok = s < len && s > 0;
        dsm[h * FS_ROWS + lane] = ok ? (rev ? xr[lane + 1] - xr[lane] : xr[lane] - xr[lane + 1]) : 0.f;
        for (int cw = 0; cw < task.count; ++cw) {
            rwl[(W + cw) * FS_RS + lane] *= __shfl_sync(0xffffffffu, pscale, cw);
        }
    };

    const int wsel = cwarp ? warp : 0;
    const int mycand = task.cand0 + wsel;
    float Fh[CPL], Fl[CPL], Gh[CPL], Gl[CPL], qh[CPL], ql[CPL], e[CPL];
    float Kh = 0.f, Kl = 0.f, kl = 0.f;  // K on the lane of the b component
#pragma unroll
    for (int u = 0; u < CPL; ++u) {
        Fh[u] = Fl[u] = Gh[u] = Gl[u] = qh[u] = ql[u] = e[u] = 0.f;
    }
    float *myFh = hFh + (size_t)wsel * FS_HIST * NCS;
    float *myFl = hFl + (size_t)wsel * FS_HIST * NCS;
    float *myGh = hGh + (size_t)wsel * FS_HIST * NCS;
    float *myGl = hGl + (size_t)wsel * FS_HIST * NCS;
    float *myK = hK + (size_t)wsel * FS_HIST * 2;
    float *myC = csum + (size_t)wsel * FS_HIST * FS_NSUM * 2;
    float *myA = cA + (size_t)wsel * FS_HIST * FS_NSUM;
    float *myE = sE + (size_t)wsel * FS_SNAP * NCS;
    float *myKL = sKL + (size_t)wsel * FS_SNAP;
    const float *myY = sycf + (size_t)wsel * (m + 1) * 2;
    const int cy = m + 1, cb = m + 2;  // the y and b components
    const float S0 = (float)mom[3 * (size_t)mycand], S1 = (float)mom[3 * (size_t)mycand + 1],
                S2 = (float)mom[3 * (size_t)mycand + 2];
    const float tolf = (float)tol, cutf = (float)cut_rel;
    float best = 0.f;
    int besti = -1;
    int flagged = 0;  // a cut the reference's f64 evaluation cannot resolve
    int nsnap = 0, nhist = 0, cur = 0;  // block-uniform
    float xbase = 0.f;                  // x at the current chunk's base (block-uniform)

    auto flush = [&]() {
        if (cwarp) {
            // per-chunk float-float sums, lane = chunk * FS_NSUM + sum
            // (0 FF, 1 FG, 2 GG, 3 Fy, 4 Gy) over the basis and candidate components
            if (lane < nhist * FS_NSUM) {
                const int ch = lane / FS_NSUM, t = lane % FS_NSUM;
                const bool ag = t == 2 || t == 4, bf = t == 0, by = t >= 3;
                const float *Ah = (ag ? myGh : myFh) + (size_t)ch * NCS;
                const float *Al = (ag ? myGl : myFl) + (size_t)ch * NCS;
                const float *Bh = (bf ? myFh : myGh) + (size_t)ch * NCS;
                const float *Bl = (bf ? myFl : myGl) + (size_t)ch * NCS;
                float sh = 0.f, sl = 0.f;
                for (int c = 0; c <= m; ++c) {
                    const float bh = by ? myY[2 * c] : Bh[c], bl = by ? myY[2 * c + 1] : Bl[c];
                    const float ah = Ah[c], al = Al[c];
                    const float p = __fmul_rn(ah, bh);
                    float pe = __fmaf_rn(ah, bh, -p);
                    pe = __fmaf_rn(ah, bl, pe);
                    pe = __fmaf_rn(al, bh, pe);
                    float s, err;
                    two_sum(sh, p, s, err);
                    sl = __fadd_rn(sl, __fadd_rn(err, pe));
                    sh = s;
                }
                myC[(ch * FS_NSUM + t) * 2] = sh;
                myC[(ch * FS_NSUM + t) * 2 + 1] = sl;
            }
            __syncwarp();
            if (lane < nhist) {
                const int ch = lane;
                const float *C = myC + ch * FS_NSUM * 2;
                const float *Fc = myFh + (size_t)ch * NCS, *Fcl = myFl + (size_t)ch * NCS;
                const float *Gc = myGh + (size_t)ch * NCS, *Gcl = myGl + (size_t)ch * NCS;
                float *A = myA + ch * FS_NSUM;
                A[0] = ff_diff(myK[2 * ch], myK[2 * ch + 1], C[0], C[1]);
                A[1] = 2.0f * ff_diff(Fc[cb], Fcl[cb], C[2], C[3]);
                A[2] = ff_diff(Gc[cb], Gcl[cb], C[4], C[5]);
                A[3] = ff_diff(C[6], C[7], Fc[cy], Fcl[cy]);
                A[4] = ff_diff(C[8], C[9], Gc[cy], Gcl[cy]);
            }
            __syncwarp();
            float sse = -1.f;
            int row = 0x7fffffff;
            if (lane < nsnap) {
                const int ch = sCh[lane];
                const float xg = sXv[lane];
                float Dh, Dl;
                two_sum(hXb[ch], -xg, Dh, Dl);
                if (rev) {
                    Dh = -Dh;
                    Dl = -Dl;
                }
                const float *Fc = myFh + (size_t)ch * NCS, *Gc = myGh + (size_t)ch * NCS;
                const float *Eg = myE + (size_t)lane * NCS;
                float Fe = 0.f, Ge = 0.f, ee = 0.f, ey = 0.f;
                for (int c = 0; c <= m; ++c) {
                    const float ec = Eg[c];
                    Fe = fmaf(Fc[c], ec, Fe);
                    Ge = fmaf(Gc[c], ec, Ge);
                    ee = fmaf(ec, ec, ee);
                    ey = fmaf(myY[2 * c], ec, ey);
                }
                const float *A = myA + ch * FS_NSUM;
                const float klg = myKL[lane];
                const float t1 = fmaf(Dh, A[2], A[1]);
                const float small = klg - 2.0f * fmaf(Dh, Ge, Fe) - ee;
                const float den = fmaf(Dh, t1, A[0]) + fmaf(Dl, fmaf(2.0f * Dh, A[2], A[1]), small);
                const float uw = fmaf(Dh, A[4], A[3]) + fmaf(Dl, A[4], ey - Eg[cy]);
                sse = den > tolf ? (uw * uw) / (den + tolf) : 0.f;
                row = srow[lane];
                // The reference forms den as (k0 + k1) - ff with k0 + k1 the
                // top-side K; when den is below cut_rel of it, that difference
                // is near the level of its f64 rounding and its value may be
                // anything: such a candidate is re-decided exactly.
                const float Kg = myK[2 * ch] + Dh * (2.0f * Fc[cb] + Dh * Gc[cb]) + klg;
                const float Kref = rev ? fmaxf(S2 - 2.0f * xg * S1 + xg * xg * S0 - Kg, 0.0f) : Kg;
                if (den < cutf * Kref) {
                    flagged = 1;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float s2 = __shfl_xor_sync(0xffffffffu, sse, o);
                const int r2 = __shfl_xor_sync(0xffffffffu, row, o);
                if (s2 > sse || (s2 == sse && r2 < row)) {
                    sse = s2;
                    row = r2;
                }
            }
            if (sse > best) {
                best = sse;
                besti = row;
            }
        }
        nsnap = 0;
        nhist = 0;
    };

    if (lwarp) {
        prefetch(0);
#pragma unroll
        for (int u = 0; u < S - 1; ++u) {
            if (u < nstages) {
                issue_bo(u);
            }
            cp_async_commit();
            prefetch(u + 1);
        }
        cp_async_wait<S - 2>();
    } else if (rwarp) {
#pragma unroll
        for (int u = 0; u < S - 1; ++u) {
            if (u < nstages) {
                issue_raw(u);
            }
            cp_async_commit();
        }
        cp_async_wait<S - 2>();
        __syncwarp();
        if (nstages > 0) {
            deltas(0);
        }
    }
    __syncthreads();
    for (int sq = 0; sq < nstages; ++sq) {
        const int sg = sq % S, h = sq & 1, s0 = sq * FS_ROWS;
        const int rows = min(FS_ROWS, len - s0);
        const bool cstart = sq % FS_CHUNK == 0;
        const bool cend = sq % FS_CHUNK == FS_CHUNK - 1 || sq == nstages - 1;
        const float *xr = sraw4 + (size_t)sg * RAW + (2 * W + 1) * FS_RS;
        // the grid rows of this stage, as bits of their offsets in it
        int gcount = 0;
        unsigned gmask = 0u;
        for (int gr = next_grid; gr < s0 + rows && gr <= last_step; gr += min_span) {
            gmask |= 1u << (gr - s0);
            ++gcount;
        }
        if (nsnap + gcount > FS_SNAP || (cstart && nhist == FS_HIST)) {
            flush();
            __syncthreads();  // snapshot and history slots are rewritten below
            if (!cstart) {
                // mid-chunk: the current chunk's carries become entry 0
                if (cwarp) {
#pragma unroll
                    for (int u = 0; u < CPL; ++u) {
                        const int c = lane + 32 * u;
                        if (c < NC) {
                            myFh[c] = myFh[(size_t)cur * NCS + c];
                            myFl[c] = myFl[(size_t)cur * NCS + c];
                            myGh[c] = myGh[(size_t)cur * NCS + c];
                            myGl[c] = myGl[(size_t)cur * NCS + c];
                        }
                    }
                    if (lane == 0) {
                        myK[0] = myK[2 * cur];
                        myK[1] = myK[2 * cur + 1];
                    }
                }
                if (threadIdx.x == 0) {
                    hXb[0] = hXb[cur];
                }
                cur = 0;
                nhist = 1;
                __syncthreads();
            }
        }
        if (cstart) {
            cur = nhist++;
            if (cwarp) {
                // carries at the start of this chunk
#pragma unroll
                for (int u = 0; u < CPL; ++u) {
                    const int c = lane + 32 * u;
                    if (c < NC) {
                        myFh[(size_t)cur * NCS + c] = Fh[u];
                        myFl[(size_t)cur * NCS + c] = Fl[u];
                        myGh[(size_t)cur * NCS + c] = Gh[u];
                        myGl[(size_t)cur * NCS + c] = Gl[u];
                    }
                    if (c == cb) {
                        myK[2 * cur] = Kh;
                        myK[2 * cur + 1] = Kl;
                    }
                }
            }
            xbase = sq == 0 ? xr[1] : xr[0];
            if (threadIdx.x == 0) {
                hXb[cur] = xbase;
            }
        }
        if (cwarp) {
            // Offsets (in floats from the start of shared memory) of this
            // stage's values: the parent b and delta d of each row, and per lane
            // where its x comes from -- the Bo row (c < m, stride MP) or one of
            // the per-row candidate arrays (candidate column, y, parent; stride
            // 1); lanes past the components read the zero word (stride 0).
            const float *smf = reinterpret_cast<const float *>(sm);
            const int rwo = (int)(L.raw / 4) + sg * RAW;
            const int bwo = rwo + warp * FS_RS;
            const int dvo = (int)(L.dsm / 4) + h * FS_ROWS;
            const int boo = (int)(L.bo / 4) + sg * FS_ROWS * MP;
            int xo[CPL], xs[CPL];
#pragma unroll
            for (int u = 0; u < CPL; ++u) {
                const int c = lane + 32 * u;
                xo[u] = c < m ? boo + c
                              : c == m ? rwo + (W + warp) * FS_RS
                                       : c == m + 1 ? rwo + 2 * W * FS_RS
                                                    : c == m + 2 ? bwo : (int)(L.zero / 4);
                xs[u] = c < m ? MP : c < NC ? 1 : 0;
            }
            int slot = nsnap;
            auto row = [&](int r) {
                const float bk = smf[bwo + r], d = smf[dvo + r];
                const float d2 = d * d, dd = 2.0f * d;
#pragma unroll
                for (int u = 0; u < CPL; ++u) {
                    const int c = lane + 32 * u;
                    const float xv = smf[xo[u] + r * xs[u]];
                    const float klc = kl + fmaf(d2, qh[u], dd * e[u]);
                    kl = c == cb ? klc : kl;
                    e[u] = fmaf(d, qh[u], e[u]);
                    float t, err;
                    two_sum(qh[u], __fmul_rn(bk, xv), t, err);
                    ql[u] = __fadd_rn(ql[u], err);
                    qh[u] = t;
                }
                if (gmask & (1u << r)) {  // a grid row: snapshot of the increments
                    float *es = myE + (size_t)slot * NCS;
#pragma unroll
                    for (int u = 0; u < CPL; ++u) {
                        const int c = lane + 32 * u;
                        if (c < NC) {
                            es[c] = e[u];
                        }
                        if (c == cb) {
                            myKL[slot] = kl;
                        }
                    }
                    if (lane == 0 && warp == 0) {
                        srow[slot] = idx(s0 + r);
                        sCh[slot] = cur;
                        sXv[slot] = xr[1 + r];
                    }
                    ++slot;
                }
            };
            if (rows == FS_ROWS) {
#pragma unroll
                for (int r = 0; r < FS_ROWS; ++r) {
                    row(r);
                }
            } else {
                for (int r = 0; r < rows; ++r) {
                    row(r);
                }
            }
            if (cend) {
                // carry to the next chunk: Dc = x_base - x_end exactly
                float Dh, Dl;
                two_sum(xbase, -xr[rows], Dh, Dl);
                if (rev) {
                    Dh = -Dh;
                    Dl = -Dl;
                }
#pragma unroll
                for (int u = 0; u < CPL; ++u) {
                    const int c = lane + 32 * u;
                    float th, tl;
                    if (c == cb) {
                        // K += Dc (2 F_b + G_b Dc) + kl, with the chunk-start F_b, G_b
                        ff_mul(Gh[u], Gl[u], Dh, Dl, th, tl);
                        ff_add(th, tl, 2.0f * Fh[u], 2.0f * Fl[u]);
                        float vh, vl;
                        ff_mul(th, tl, Dh, Dl, vh, vl);
                        ff_add(Kh, Kl, vh, vl);
                        ff_add(Kh, Kl, kl, 0.0f);
                    }
                    ff_mul(Gh[u], Gl[u], Dh, Dl, th, tl);
                    ff_add(Fh[u], Fl[u], th, tl);
                    ff_add(Fh[u], Fl[u], e[u], 0.0f);
                    ff_add(Gh[u], Gl[u], qh[u], ql[u]);
                    qh[u] = ql[u] = e[u] = 0.f;
                }
                kl = 0.f;
            }
        } else if (lwarp) {
            if (sq + S - 1 < nstages) {
                issue_bo(sq + S - 1);
            }
            cp_async_commit();
            prefetch(sq + S);
            cp_async_wait<S - 2>();
        } else if (rwarp) {
            if (sq + S - 1 < nstages) {
                issue_raw(sq + S - 1);
            }
            cp_async_commit();
            cp_async_wait<S - 2>();
            __syncwarp();
            if (sq + 1 < nstages) {
                deltas(sq + 1);
            }
        }
        nsnap += gcount;
        next_grid += gcount * min_span;
        __syncthreads();
    }
    if (nsnap > 0) {
        flush();
    }
    flagged = __any_sync(0xffffffffu, flagged);
    if (cwarp && lane == 0) {
        hsse[(size_t)mycand * 2 + task.dir] = (double)best;
        hrow[(size_t)mycand * 2 + task.dir] = besti >= 0 ? pk[besti] : -1;
        hflag[(size_t)mycand * 2 + task.dir] = flagged;
    }
}

}  // namespace

int fast_ksplit(int n) { return std::max(1, std::min(64, n / 2048)); }

int fast_sweep_mid(int head, int tail, int n)
{
    return std::max(0, std::min((head + tail) / 2, n - 1));
}

size_t fast_norm_part_bytes(size_t n, size_t P)
{
    return sizeof(double) * 2 * std::max<size_t>(P, 1) * ceil_div(std::max<size_t>(n, 1), FN_ROWS);
}

void fast_norms_rows(cudaStream_t st, const float *Bx, size_t ldr, int n, const float *y,
                     double tol, int P, double *part, double *s, double *ybx,
                     long long *launches)
{
    const int nch = (int)ceil_div((size_t)std::max(n, 1), FN_ROWS);
    const dim3 g((unsigned)ceil_div((size_t)P, 32), (unsigned)nch);
    k_fast_norms_rows<<<g, 256, 0, st>>>(Bx, ldr, n, y, P, part);
    LAUNCH_CHECK();
    k_fast_norms_rows_done<<<(unsigned)ceil_div((size_t)P, 256), 256, 0, st>>>(part, nch, P, tol,
                                                                             s, ybx);
    LAUNCH_CHECK();
    *launches += 2;
}

void fast_parent_moments(cudaStream_t st, const FillSrc &src, int n, int P, double *mom,
                         long long *launches)
{
    k_parent_moments<<<(unsigned)P, 256, 0, st>>>(src, n, mom);
    LAUNCH_CHECK();
    *launches += 1;
}

void fast_to_rows(cudaStream_t st, const float *Bc, int n, int P, float *Br, size_t ldr,
                  long long *launches)
{
    const dim3 g((unsigned)ceil_div((size_t)n, 32), (unsigned)ceil_div((size_t)P, 32));
    k_fast_to_rows<<<g, dim3(32, 8), 0, st>>>(Bc, n, P, Br, ldr);
    LAUNCH_CHECK();
    *launches += 1;
}

void fast_norms_moments(cudaStream_t st, const float *Bx, int n, const float *y, double tol,
                        const FillSrc &src, int P, double *s, double *ybx, double *mom,
                        long long *launches)
{
    k_fast_norms<<<(unsigned)P, 256, 0, st>>>(Bx, n, y, tol, s, ybx);
    LAUNCH_CHECK();
    k_parent_moments<<<(unsigned)P, 256, 0, st>>>(src, n, mom);
    LAUNCH_CHECK();
    *launches += 2;
}

void fast_project(cudaStream_t st, const FillSrc &src, const float *BoC, int n, int m, int P,
                  const float *y, double tol, const FastScratch &ws, long long *launches)
{
    if (P <= 0) {
        return;
    }
    verify(m >= 1, "the fast projection needs at least one basis column");
    const int ks = fast_ksplit(n);
    const int rps = (int)round_up(ceil_div(n, ks), FT_ROWS);
    const size_t tcount = (size_t)P * std::max(m, 1);
    verify(ceil_div(P, 32) <= 2147483647u && ceil_div(m, 32) <= 65535 && ks <= 65535,
           "fast projection grid out of range", 2);
    const size_t psmem = sizeof(float) * FP_COLS * std::max(m, 1);
    verify(psmem <= 227 * 1024, "the fast projection supports at most 900 basis functions");
    verify(ceil_div(P, FP_COLS) <= 65535, "too many candidate columns for one launch", 2);
    StoredSrc stored{ws.Bx, (size_t)n, nullptr};
    for (int pass = 0; pass < 2; ++pass) {
        const dim3 g1((unsigned)ceil_div(P, 32), (unsigned)ceil_div(m, 32), (unsigned)ks);
        if (pass == 0) {
            k_fast_tgemm<FillSrc><<<g1, FT_THREADS, 0, st>>>(src, BoC, n, m, P, rps, ws.Tp);
        } else {
            k_fast_tgemm<StoredSrc><<<g1, FT_THREADS, 0, st>>>(stored, BoC, n, m, P, rps, ws.Tp);
        }
        LAUNCH_CHECK();
        k_fast_treduce<<<(unsigned)ceil_div(tcount, 256), 256, 0, st>>>(ws.Tp, ks, tcount, ws.T);
        LAUNCH_CHECK();
        const dim3 g2((unsigned)ceil_div(n, FP_ROWS), (unsigned)ceil_div(P, FP_COLS));
        if (pass == 0) {
            if (psmem > 48 * 1024) {
                allow_smem(k_fast_project<FillSrc>, psmem);
            }
            k_fast_project<FillSrc><<<g2, FP_THREADS, psmem, st>>>(src, BoC, n, m, P, ws.T, ws.Bx);
        } else {
            if (psmem > 48 * 1024) {
                allow_smem(k_fast_project<StoredSrc>, psmem);
            }
            k_fast_project<StoredSrc><<<g2, FP_THREADS, psmem, st>>>(stored, BoC, n, m, P, ws.T,
                                                                   ws.Bx);
        }
        LAUNCH_CHECK();
        *launches += 3;
    }
    fast_norms_moments(st, ws.Bx, n, y, tol, src, P, ws.s, ws.ybx, ws.mom, launches);
}

static size_t fast_sweep_smem(int m, int w, int stages) { return FastSweepSmem(m, w, stages).total; }

// Resident blocks per SM for W candidate warps and S stages: shared memory
// (228 KB per SM, 1 KB of it reserved per block) and registers.
static int fast_sweep_regs();

// The sweep is compiled for two of its largest blocks per SM (at most ~100
// registers): measured on the n = 1e6 fit, the sweep phase went 172 -> 132 ms
// a step at 13 basis columns and 422 -> 328 ms at 50 against the uncapped
// kernel; a cap for three blocks (~64 registers) spilled and was slower.
constexpr int FS_RB = 2;

static int fast_sweep_bps(int m, int w, int stages)
{
    const size_t sm = fast_sweep_smem(m, w, stages) + 1024;
    const int by_smem = (int)((228 * 1024) / sm);
    const int by_regs = 65536 / (fast_sweep_regs() * 32 * (w + 2));
    return std::max(0, std::min(std::min(by_smem, by_regs), 32));
}

// Registers per thread of the sweep kernel (the instances differ little).
static int fast_sweep_regs()
{
    static const int regs = [] {
        cudaFuncAttributes fa;
        const cudaError_t e = cudaFuncGetAttributes(&fa, k_fast_sweep<1, 4, FS_RB>);
        const int r = e == cudaSuccess ? std::max(fa.numRegs, 32) : 168;
        cudaGetLastError();
        return r;
    }();
    return regs;
}

// The stage depth: the deepest ring (4, 3 or 2 stages of 32 rows) that lets
// as many blocks reside as the shallowest. With two stages the loaders wait
// for the stage they have just issued; with three the load of a stage has a
// whole stage of compute to land in.
static int fast_sweep_stages(int m, int w)
{
    const int b2 = fast_sweep_bps(m, w, 2);
    return fast_sweep_bps(m, w, 4) >= b2 ? 4 : fast_sweep_bps(m, w, 3) >= b2 ? 3 : 2;
}

int fast_sweep_warps(int m, const std::vector<int> &group_sizes)
{
    // Each candidate warp walks half the sorted rows one after another, so the
    // launch takes about (waves of blocks) x (one walk): choose the block
    // width with the fewest waves on 152 SMs, and among those the widest
    // (fewer loader warps per candidate).
    int best_w = 1;
    long best_waves = -1;
    for (int w : {FS_MAXW, 4, 2, 1}) {
        if (fast_sweep_smem(m, w, 2) > 227 * 1024) {
            continue;
        }
        const int bps = fast_sweep_bps(m, w, fast_sweep_stages(m, w));
        if (bps == 0) {
            continue;
        }
        long blocks = 0;
        for (int g : group_sizes) {
            blocks += 2 * ((g + w - 1) / w);
        }
        const long waves = (blocks + 152L * bps - 1) / (152L * bps);
        if (best_waves < 0 || waves < best_waves) {
            best_waves = waves;
            best_w = w;
        }
    }
    return best_w;
}

void fast_sweep(cudaStream_t st, const FastTaskRec *tasks, int ntasks, const int *perm,
                const float *xsort, const float *ysort, const FastSweepCols &cols,
                const float *BoR, size_t ldbo, const double *ybo, const double *ybx,
                const double *mom, int n, int m, int head, int tail, int min_span, double tol,
                double cut_rel, double *hsse, int *hrow, int *hflag, int warps_per_block,
                long long *launches)
{
    if (ntasks <= 0) {
        return;
    }
    const int warps = warps_per_block;
    verify(warps >= 1 && warps <= FS_MAXW, "sweep block size out of range", 2);
    const int stages = fast_sweep_stages(m, warps);
    const size_t smem = fast_sweep_smem(m, warps, stages);
    verify(smem <= 227 * 1024, "too many basis functions for the fast hinge sweep");
    const int nc = m + 3;
    const int mid = fast_sweep_mid(head, tail, n);
#define LAUNCH_FS_RB(CPL, S, RB)                                                               \
    do {                                                                                       \
        allow_smem(k_fast_sweep<CPL, S, RB>, smem);                                            \
        k_fast_sweep<CPL, S, RB><<<ntasks, 32 * (warps + 2), smem, st>>>(                      \
            reinterpret_cast<const FastTask *>(tasks), perm, xsort, ysort, cols, BoR, ldbo,    \
            ybo, ybx, mom, n, m, head, tail, mid, min_span, tol, cut_rel, hsse, hrow, hflag);  \
    } while (0)
#define LAUNCH_FS_CPL(CPL)                   \
    do {                                     \
        if (stages == 4) {                   \
            LAUNCH_FS_RB(CPL, 4, FS_RB);     \
        } else if (stages == 3) {            \
            LAUNCH_FS_RB(CPL, 3, FS_RB);     \
        } else {                             \
            LAUNCH_FS_RB(CPL, 2, FS_RB);     \
        }                                    \
    } while (0)
    if (nc <= 32) {
        LAUNCH_FS_CPL(1);
    } else if (nc <= 64) {
        LAUNCH_FS_CPL(2);
    } else if (nc <= 128) {
        LAUNCH_FS_CPL(4);
    } else if (nc <= 256) {
        LAUNCH_FS_CPL(8);
    } else {
        throw Error(1, "the fast hinge sweep supports at most 253 basis functions");
    }
#undef LAUNCH_FS_CPL
#undef LAUNCH_FS_RB
    LAUNCH_CHECK();
    *launches += 1;
}

}  // namespace mgpu
