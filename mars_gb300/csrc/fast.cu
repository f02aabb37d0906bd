// Fast (ranking) pass of the mixed-precision forward pass.
//
// Projection: FP32 split-K GEMMs (T = Bo^T v, then v - Bo T), applied twice
// so the second pass re-orthogonalises the first one's residual (the role of
// the reference's DGKS step, kernels.cc:384-395), then FP32 norms with FP64
// block sums.
//
// Hinge sweep: the reference's recurrences (marsalgo.cc:576-649 with
// covariates_impl :91-151) in chunks of FS_ROWS sorted rows: inside a chunk the
// increments are FP32, across chunks the running values are carried in FP64:
//   g_c(i) = G_c + q_c(i)
//   f_c(i) = F_c + G_c D(i) + e_c(i)      (D(i): sum of the chunk's deltas to row i)
// with e_c += d q_c, q_c += b x_c in FP32. Besides the basis columns and the
// candidate column, two more components carry the scalar recurrences: x = y
// (g = vb, f = w) and x = b (g = b2, f = bd), and K = k0 + k1 follows as
//   K(i) = K + 2 F_b D(i) + G_b D(i)^2 + kl(i),   kl += d^2 q_b + 2 d e_b.
// A grid row stores only the FP32 increments; the scores are rebuilt in FP64
// from the carries, 32 grid rows at a time (lane = grid row).
#include "fast.cuh"

#include <algorithm>

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
// squared norm of the candidate column x b).
__global__ void __launch_bounds__(256) k_parent_moments(FillSrc src, int n, double *__restrict__ mom)
{
    __shared__ double red[3][8];
    const int j = blockIdx.x, t = threadIdx.x;
    const int xc = src.cand_x[j];
    const float *bcol = src.B + (size_t)src.cand_b[j] * src.ldB;
    const float *xcol = src.X + (size_t)xc * src.ldX;
    const float sx = src.s[xc];
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int i = t; i < n; i += 256) {
        const double b = bcol[i], x = (double)(xcol[i] * sx);
        const double b2 = b * b;
        a0 += b2;
        a1 += b2 * x;
        a2 += b2 * x * x;
    }
    a0 = warp_sum(a0);
    a1 = warp_sum(a1);
    a2 = warp_sum(a2);
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

// ---------------------------------------------------------------------------
// Chunked sweep. Block = one input column, one direction and up to W
// candidates (warps 0..W-1, lane = component) plus two loader warps that stage
// each chunk with cp.async: warp W the gathered f32 Bo rows (16 bytes per
// lane), warp W+1, lanes over rows, the sorted parent and candidate values, y
// and x, then the f32 deltas and their f64 running sums within the chunk
// (copies in flight are limited per warp, so the staging is split).
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
// Scoring, 32 grid rows at a time: first the per-chunk f64 sums
// FF = sum F_c^2, FG = sum F_c G_c, GG = sum G_c^2, Fy = sum F_c yc_c,
// Gy = sum G_c yc_c (one lane per chunk and sum), then per grid row (one lane
// each), with f32 cross terms against f32 copies of the carries,
//   ff = FF + 2D FG + D^2 GG + 2 (sum F_c e_c + D sum G_c e_c) + sum e_c^2
//   fy = Fy + D Gy + sum e_c yc_c,   w = F_y + D G_y + e_y,
//   K  = K + 2 F_b D + G_b D^2 + kl.
// ---------------------------------------------------------------------------
constexpr int FS_ROWS = 32, FS_SNAP = 32, FS_HIST = 6, FS_NSUM = 5, FS_MAXW = 8;

using FastTask = FastTaskRec;  // dir 0: forward (first half of the cuts), 1: mirror (second half)

struct FastSweepSmem {
    size_t hF, hG, hK, cst, sD, ybo, dpre, hFf, hGf, sE, sKL, sCh, srow, sXv, ycf, bo, raw, dsm,
        total;
    __host__ __device__ FastSweepSmem(int m, int W, int S)
    {
        const int nc = m + 3;
        size_t o = 0;
        hF = o;  // [W][FS_HIST][nc] f64 carries at chunk starts
        o += 8 * (size_t)W * FS_HIST * nc;
        hG = o;
        o += 8 * (size_t)W * FS_HIST * nc;
        hK = o;  // [W][FS_HIST]
        o += 8 * (size_t)W * FS_HIST;
        cst = o;  // [W][FS_HIST][FS_NSUM] per-chunk f64 sums
        o += 8 * (size_t)W * FS_HIST * FS_NSUM;
        sD = o;  // [FS_SNAP] f64 D at the grid row
        o += 8 * FS_SNAP;
        ybo = o;  // [m + 1] f64 (component m: the candidate's ybx, per warp below)
        o += 8 * ((size_t)m + 1);
        dpre = o;  // [2][FS_ROWS] f64 running delta sums of a chunk
        o += 8 * 2 * FS_ROWS;
        hFf = o;  // [W][FS_HIST][nc] f32 copies of the carries
        o += 4 * (size_t)W * FS_HIST * nc;
        hGf = o;
        o += 4 * (size_t)W * FS_HIST * nc;
        sE = o;  // [W][FS_SNAP][nc] f32 increments e at grid rows
        o += 4 * (size_t)W * FS_SNAP * nc;
        sKL = o;  // [W][FS_SNAP]
        o += 4 * (size_t)W * FS_SNAP;
        sCh = o;  // [FS_SNAP] chunk history index of the grid row
        o += 4 * FS_SNAP;
        srow = o;  // [FS_SNAP] sorted row of the grid row
        o += 4 * FS_SNAP;
        sXv = o;  // [FS_SNAP] f32 x (the knot) of the grid row
        o += 4 * FS_SNAP;
        ycf = o;  // [W][m + 1] f32 y coefficients (ybo, then ybx)
        o += 4 * (size_t)W * (m + 1);
        o = (o + 15) / 16 * 16;  // 16-byte cp.async destinations
        bo = o;  // [S][FS_ROWS][mp] f32, row stride mp = m rounded up to 4
        o += 4 * (size_t)S * FS_ROWS * ((m + 3) / 4 * 4);
        raw = o;  // [S][(2W + 1) * FS_ROWS + FS_ROWS + 1] f32: B, Bx per candidate, y, x
        o += 4 * (size_t)S * ((2 * W + 1) * FS_ROWS + FS_ROWS + 1);
        dsm = o;  // [2][FS_ROWS] f32 deltas
        o += 4 * 2 * FS_ROWS;
        total = (o + 15) / 16 * 16;
    }
};

template <int CPL, int S>
__global__ void __launch_bounds__(32 * (FS_MAXW + 2), 1)
    k_fast_sweep(const FastTask *__restrict__ tasks, const int *__restrict__ perm,
                 const float *__restrict__ xsort, const float *__restrict__ ysort,
                 const float *__restrict__ bs, const float *__restrict__ bxs,
                 const float *__restrict__ BoR, size_t ldbo, const double *__restrict__ ybo,
                 const double *__restrict__ ybx, const double *__restrict__ mom, int n, int m,
                 int head, int tail, int mid, int min_span, double tol, double cut_rel,
                 double *__restrict__ hsse, int *__restrict__ hrow, int *__restrict__ hflag)
{
    extern __shared__ __align__(16) unsigned char sm[];
    const int W = (blockDim.x >> 5) - 2;  // candidate warps; then the two loaders
    const int NC = m + 3;  // basis columns, candidate, y, b
    const int U = (m + 3) / 4, MP = 4 * U;  // 16-byte units per Bo row, padded row stride
    const int RAW = (2 * W + 1) * FS_ROWS + FS_ROWS + 1;
    const FastSweepSmem L(m, W, S);
    double *hF = reinterpret_cast<double *>(sm + L.hF);
    double *hG = reinterpret_cast<double *>(sm + L.hG);
    double *hK = reinterpret_cast<double *>(sm + L.hK);
    double *cst = reinterpret_cast<double *>(sm + L.cst);
    double *sD = reinterpret_cast<double *>(sm + L.sD);
    double *sybo = reinterpret_cast<double *>(sm + L.ybo);
    double *dpre = reinterpret_cast<double *>(sm + L.dpre);
    float *hFf = reinterpret_cast<float *>(sm + L.hFf);
    float *hGf = reinterpret_cast<float *>(sm + L.hGf);
    float *sE = reinterpret_cast<float *>(sm + L.sE);
    float *sKL = reinterpret_cast<float *>(sm + L.sKL);
    int *sCh = reinterpret_cast<int *>(sm + L.sCh);
    int *srow = reinterpret_cast<int *>(sm + L.srow);
    float *sXv = reinterpret_cast<float *>(sm + L.sXv);
    float *sycf = reinterpret_cast<float *>(sm + L.ycf);
    float *sbo = reinterpret_cast<float *>(sm + L.bo);
    float *sraw4 = reinterpret_cast<float *>(sm + L.raw);
    float *dsm = reinterpret_cast<float *>(sm + L.dsm);

    const FastTask task = tasks[blockIdx.x];
    const bool rev = task.dir != 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool cwarp = warp < task.count;
    const bool lwarp = warp == W;      // loader of the Bo rows
    const bool rwarp = warp == W + 1;  // loader of the per-candidate arrays, y, x
    const int *pk = perm + (size_t)task.xcol * n;
    const float *xs = xsort + (size_t)task.xcol * n;
    const float *ys = ysort + (size_t)task.xcol * n;
    const float *bsb = bs + (size_t)task.cand0 * n;
    const float *bxb = bxs + (size_t)task.cand0 * n;
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        sybo[c] = ybo[c];
    }
    for (int e = threadIdx.x; e < W * (m + 1); e += blockDim.x) {
        const int w = e / (m + 1), c = e % (m + 1);
        sycf[e] = (float)(c < m ? ybo[c] : (w < task.count ? ybx[task.cand0 + w] : 0.0));
    }
    __syncthreads();

    // Processing step s visits sorted row idx(s); the task's cuts are the grid
    // rows g = head + 1 + k min_span <= tail - 1 on its side of mid.
    const int len = rev ? n - 1 - mid : mid + 1;
    auto idx = [&](int s) { return rev ? n - 1 - s : s; };
    const long g_last = tail - 1 >= head + 1
                            ? (long)head + 1 + (long)((tail - 1 - (head + 1)) / min_span) * min_span
                            : -1;
    long next_grid, last_step;  // in processing steps
    if (!rev) {
        next_grid = (long)head + 1;
        last_step = g_last < 0 ? -1 : (g_last < (long)mid ? g_last : (long)mid);
    } else {
        next_grid = g_last < 0 ? (long)len : (long)n - 1 - g_last;  // largest grid row first
        last_step = g_last < 0 ? -1 : (long)n - 1 - (mid + 1);
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
        for (int cw = 0; cw < task.count; ++cw) {
            cp_async4(rw + cw * FS_ROWS + lane, bsb + (size_t)cw * n + i, ok);
            cp_async4(rw + (W + cw) * FS_ROWS + lane, bxb + (size_t)cw * n + i, ok);
        }
        cp_async4(rw + 2 * W * FS_ROWS + lane, ys + i, ok);
        cp_async4(rw + (2 * W + 1) * FS_ROWS + 1 + lane, xs + i, ok);
        if (lane == 0) {
            cp_async4(rw + (2 * W + 1) * FS_ROWS, xs + (s0 > 0 ? idx(s0 - 1) : 0), s0 > 0);
        }
    };
    // Stage sq (landed): f32 deltas and their f64 running sums (lanes = rows).
    auto deltas = [&](int sq) {
        const float *xr = sraw4 + (size_t)(sq % S) * RAW + (2 * W + 1) * FS_ROWS;
        const int h = sq & 1, s = sq * FS_ROWS + lane;
        const bool ok = s < len && s > 0;
        const float d = ok ? (rev ? xr[lane + 1] - xr[lane] : xr[lane] - xr[lane + 1]) : 0.f;
        // running sum of the chunk's deltas through this row: telescoped, the
        // f64 difference of the x at the chunk's base and at the row
        const float base = sq == 0 ? xr[1] : xr[0];
        const double run = rev ? (double)xr[lane + 1] - (double)base
                               : (double)base - (double)xr[lane + 1];
        dsm[h * FS_ROWS + lane] = d;
        dpre[h * FS_ROWS + lane] = run;
    };

    const int wsel = cwarp ? warp : 0;
    const int mycand = task.cand0 + wsel;
    double F[CPL], G[CPL], K = 0.0;
    float e[CPL], q[CPL], kl = 0.f;
#pragma unroll
    for (int u = 0; u < CPL; ++u) {
        F[u] = 0.0;
        G[u] = 0.0;
        e[u] = 0.f;
        q[u] = 0.f;
    }
    double *myF = hF + (size_t)wsel * FS_HIST * NC;
    double *myG = hG + (size_t)wsel * FS_HIST * NC;
    float *myFf = hFf + (size_t)wsel * FS_HIST * NC;
    float *myGf = hGf + (size_t)wsel * FS_HIST * NC;
    double *myK = hK + (size_t)wsel * FS_HIST;
    double *myC = cst + (size_t)wsel * FS_HIST * FS_NSUM;
    float *myE = sE + (size_t)wsel * FS_SNAP * NC;
    float *myKL = sKL + (size_t)wsel * FS_SNAP;
    const float *myY = sycf + (size_t)wsel * (m + 1);
    const double ybx_c = ybx[mycand];
    const int cb = m + 2;  // the b component (K lives on its lane)
    const double S0 = mom[3 * (size_t)mycand], S1 = mom[3 * (size_t)mycand + 1],
                 S2 = mom[3 * (size_t)mycand + 2];
    double best = 0.0;
    int besti = -1;
    int flagged = 0;  // a cut the reference's f64 evaluation cannot resolve
    int nsnap = 0, nhist = 0;  // block-uniform

    auto flush = [&]() {
        if (cwarp) {
            // per-chunk f64 sums, lane = chunk * FS_NSUM + sum
            if (lane < nhist * FS_NSUM) {
                const int ch = lane / FS_NSUM, t = lane % FS_NSUM;
                const double *Fh = myF + (size_t)ch * NC, *Gh = myG + (size_t)ch * NC;
                double acc = 0.0;
                for (int c = 0; c <= m; ++c) {
                    // t: 0 FF, 1 FG, 2 GG, 3 Fy, 4 Gy
                    const double yc = c < m ? sybo[c] : ybx_c;
                    const double a = (t == 2 || t == 4) ? Gh[c] : Fh[c];
                    const double b = t == 0 ? Fh[c] : (t == 1 || t == 2) ? Gh[c] : yc;
                    acc = fma(a, b, acc);
                }
                myC[ch * FS_NSUM + t] = acc;
            }
            __syncwarp();
            double sse = -1.0;
            int row = 0x7fffffff;
            if (lane < nsnap) {
                const int ch = sCh[lane];
                const double D = sD[lane];
                const float *Ff = myFf + (size_t)ch * NC, *Gf = myGf + (size_t)ch * NC;
                const float *Eg = myE + (size_t)lane * NC;
                float Fe = 0.f, Ge = 0.f, ee = 0.f, ey = 0.f;
                for (int c = 0; c <= m; ++c) {
                    const float ec = Eg[c];
                    Fe = fmaf(Ff[c], ec, Fe);
                    Ge = fmaf(Gf[c], ec, Ge);
                    ee = fmaf(ec, ec, ee);
                    ey = fmaf(myY[c], ec, ey);
                }
                const double *C = myC + (size_t)ch * FS_NSUM;
                const double *Fh = myF + (size_t)ch * NC, *Gh = myG + (size_t)ch * NC;
                const double ff = C[0] + D * (2.0 * C[1] + D * C[2]) +
                                  2.0 * ((double)Fe + D * (double)Ge) + (double)ee;
                const double fy = C[3] + D * C[4] + (double)ey;
                const double w = fma(Gh[m + 1], D, Fh[m + 1]) + (double)Eg[m + 1];
                const double Kg = myK[ch] + D * (2.0 * Fh[cb] + D * Gh[cb]) + (double)myKL[lane];
                const double uw = fy - w;
                const double den = Kg - ff;
                sse = den > tol ? (uw * uw) / (den + tol) : 0.0;
                row = srow[lane];
                // The reference forms den as (k0 + k1) - ff with k0 + k1 the
                // top-side K; when den is below cut_rel of it, that difference
                // is near the level of its f64 rounding and its value may be
                // anything: such a candidate is re-decided exactly.
                const double t = (double)sXv[lane];
                const double Kref = rev ? fmax(S2 - 2.0 * t * S1 + t * t * S0 - Kg, 0.0) : Kg;
                if (den < cut_rel * Kref) {
                    flagged = 1;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double s2 = __shfl_xor_sync(0xffffffffu, sse, o);
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
        int gcount = 0;
        for (long gr = next_grid; gr < s0 + rows && gr <= last_step; gr += min_span) {
            ++gcount;
        }
        if (nsnap + gcount > FS_SNAP || nhist == FS_HIST) {
            flush();
            __syncthreads();  // snapshot and history slots are rewritten below
        }
        if (cwarp) {
            // carries at the start of this chunk (f64, and f32 copies)
#pragma unroll
            for (int u = 0; u < CPL; ++u) {
                const int c = lane + 32 * u;
                if (c < NC) {
                    myF[(size_t)nhist * NC + c] = F[u];
                    myG[(size_t)nhist * NC + c] = G[u];
                    myFf[(size_t)nhist * NC + c] = (float)F[u];
                    myGf[(size_t)nhist * NC + c] = (float)G[u];
                }
                if (c == cb) {
                    myK[nhist] = K;
                }
            }
            const float *rw = sraw4 + (size_t)sg * RAW;
            const float *bw = rw + warp * FS_ROWS;
            const float *dv = dsm + h * FS_ROWS;
            const float *rowb = sbo + (size_t)sg * FS_ROWS * MP;
            long ng = next_grid;
            int slot = nsnap;
            // Per lane, where its x comes from: the Bo row (c < m) or one of the
            // per-row candidate arrays (candidate column, y, parent); the same
            // address arithmetic for every row, no per-row selects.
            int xoff[CPL];
            bool xrow[CPL];
#pragma unroll
            for (int u = 0; u < CPL; ++u) {
                const int c = lane + 32 * u;
                xrow[u] = c < m;
                xoff[u] = c < m ? c
                                : c == m ? (W + warp) * FS_ROWS
                                         : c == m + 1 ? 2 * W * FS_ROWS : warp * FS_ROWS;
            }
            int r = 0;
            while (r < rows) {
                // rows up to and including the next grid row of this stage run
                // without a branch; the snapshot follows
                const bool grid_here = ng <= last_step && ng < (long)s0 + rows;
                const int rend = grid_here ? (int)(ng - s0) + 1 : rows;
#pragma unroll 4
                for (; r < rend; ++r) {
                    const float bk = bw[r], d = dv[r];
                    const float *rowp = rowb + r * MP;
#pragma unroll
                    for (int u = 0; u < CPL; ++u) {
                        const int c = lane + 32 * u;
                        const float xv = xrow[u] ? rowp[xoff[u]] : (c < NC ? rw[xoff[u] + r] : 0.f);
                        const float klc = fmaf(d * d, q[u], fmaf(2.0f * d, e[u], kl));
                        kl = c == cb ? klc : kl;
                        e[u] = fmaf(d, q[u], e[u]);
                        q[u] = fmaf(bk, xv, q[u]);
                    }
                }
                if (grid_here) {
                    const int rg = rend - 1;
                    ng += min_span;
                    float *es = myE + (size_t)slot * NC;
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
                        srow[slot] = idx(s0 + rg);
                        sCh[slot] = nhist;
                        sD[slot] = dpre[h * FS_ROWS + rg];
                        sXv[slot] = rw[(2 * W + 1) * FS_ROWS + 1 + rg];
                    }
                    ++slot;
                }
            }
            // carry to the next chunk start (f64)
            const double Dc = dpre[h * FS_ROWS + rows - 1];
#pragma unroll
            for (int u = 0; u < CPL; ++u) {
                const int c = lane + 32 * u;
                if (c == cb) {
                    K = K + Dc * (2.0 * F[u] + Dc * G[u]) + (double)kl;
                }
                F[u] = fma(G[u], Dc, F[u]) + (double)e[u];
                G[u] = G[u] + (double)q[u];
                e[u] = 0.f;
                q[u] = 0.f;
            }
            kl = 0.f;
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
        nhist += 1;
        next_grid += (long)gcount * min_span;
        __syncthreads();
    }
    if (nsnap > 0) {
        flush();
    }
    flagged = __any_sync(0xffffffffu, flagged);
    if (cwarp && lane == 0) {
        hsse[(size_t)mycand * 2 + task.dir] = best;
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
                CUDA_CHECK(cudaFuncSetAttribute(k_fast_project<FillSrc>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)psmem));
            }
            k_fast_project<FillSrc><<<g2, FP_THREADS, psmem, st>>>(src, BoC, n, m, P, ws.T, ws.Bx);
        } else {
            if (psmem > 48 * 1024) {
                CUDA_CHECK(cudaFuncSetAttribute(k_fast_project<StoredSrc>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)psmem));
            }
            k_fast_project<StoredSrc><<<g2, FP_THREADS, psmem, st>>>(stored, BoC, n, m, P, ws.T,
                                                                   ws.Bx);
        }
        LAUNCH_CHECK();
        *launches += 3;
    }
    k_fast_norms<<<(unsigned)P, 256, 0, st>>>(ws.Bx, n, y, tol, ws.s, ws.ybx);
    LAUNCH_CHECK();
    k_parent_moments<<<(unsigned)P, 256, 0, st>>>(src, n, ws.mom);
    LAUNCH_CHECK();
    *launches += 2;
}

static size_t fast_sweep_smem(int m, int w, int stages) { return FastSweepSmem(m, w, stages).total; }

int fast_sweep_warps(int m, int candidates)
{
    int w = candidates <= 4 * 152 ? 4 : FS_MAXW;
    while (w > 1 && fast_sweep_smem(m, w, 2) > 200 * 1024) {
        --w;
    }
    return w;
}

void fast_sweep(cudaStream_t st, const FastTaskRec *tasks, int ntasks, const int *perm,
                const float *xsort, const float *ysort, const float *bs, const float *bxs,
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
    const int stages = fast_sweep_smem(m, warps, 4) <= 200 * 1024 ? 4 : 2;
    const size_t smem = fast_sweep_smem(m, warps, stages);
    verify(smem <= 227 * 1024, "too many basis functions for the fast hinge sweep");
    const int nc = m + 3;
    const int mid = fast_sweep_mid(head, tail, n);
#define LAUNCH_FS(CPL, S)                                                                      \
    do {                                                                                       \
        CUDA_CHECK(cudaFuncSetAttribute(k_fast_sweep<CPL, S>,                                  \
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,           \
                                        (int)smem));                                           \
        k_fast_sweep<CPL, S><<<ntasks, 32 * (warps + 2), smem, st>>>(                          \
            reinterpret_cast<const FastTask *>(tasks), perm, xsort, ysort, bs, bxs, BoR, ldbo, \
            ybo, ybx, mom, n, m, head, tail, mid, min_span, tol, cut_rel, hsse, hrow, hflag);  \
    } while (0)
#define LAUNCH_FS_CPL(CPL)      \
    do {                        \
        if (stages == 4) {      \
            LAUNCH_FS(CPL, 4);  \
        } else {                \
            LAUNCH_FS(CPL, 2);  \
        }                       \
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
#undef LAUNCH_FS
    LAUNCH_CHECK();
    *launches += 1;
}

}  // namespace mgpu
