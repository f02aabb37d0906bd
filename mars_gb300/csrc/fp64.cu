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
// T = Bo^T Bx with every entry accumulated over the rows in order
// i = 0..n-1 by one fused-multiply-add chain, which is the reference's order
// (kernels.cc:327-335: tc[k] += bo_row[k] * bx[i], rows outermost). The block
// tile is KT components x (128 / KT) columns, one accumulator per thread; the
// rows are staged 32 at a time in shared memory.
// ---------------------------------------------------------------------------
constexpr int TG_ROWS = 32, TG_THREADS = 128;

template <class Src, int KT>
__global__ void __launch_bounds__(TG_THREADS)
    k_tgemm(Src src, const float *__restrict__ Bo, size_t ldbo, int n, int m, int P,
            double *__restrict__ T)
{
    constexpr int JT = TG_THREADS / KT;
    __shared__ double sBo[2][TG_ROWS][KT + 1];
    __shared__ double sV[2][TG_ROWS][JT + 1];
    const int t = threadIdx.x, kk = t % KT, jj = t / KT;
    const int k0 = blockIdx.x * KT, j0 = blockIdx.y * JT;
    // Rows of the next tile are loaded into registers before the current tile's
    // chain steps, and stored to the other half after them.
    constexpr int NB = (TG_ROWS * KT + TG_THREADS - 1) / TG_THREADS;
    constexpr int NV = (TG_ROWS * JT + TG_THREADS - 1) / TG_THREADS;
    double rb[NB], rv[NV];
    auto fetch = [&](int r0) {
        const int rows = min(TG_ROWS, n - r0);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int e = t + q * TG_THREADS;
            const int rr = e / KT, cc = e % KT;
            rb[q] = (e < TG_ROWS * KT && rr < rows && k0 + cc < m)
                        ? (double)Bo[(size_t)(r0 + rr) * ldbo + k0 + cc] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const int e = t + q * TG_THREADS;
            const int rr = e % TG_ROWS, cj = e / TG_ROWS;
            rv[q] = (e < TG_ROWS * JT && rr < rows && j0 + cj < P)
                        ? (double)src((size_t)(r0 + rr), j0 + cj) : 0.0;
        }
    };
    auto put = [&](int h) {
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int e = t + q * TG_THREADS;
            if (e < TG_ROWS * KT) {
                sBo[h][e / KT][e % KT] = rb[q];
            }
        }
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const int e = t + q * TG_THREADS;
            if (e < TG_ROWS * JT) {
                sV[h][e % TG_ROWS][e / TG_ROWS] = rv[q];
            }
        }
    };
    double acc = 0.0;
    if (n > 0) {
        fetch(0);
        put(0);
    }
    __syncthreads();
    int h = 0;
    for (int r0 = 0; r0 < n; r0 += TG_ROWS, h ^= 1) {
        const int rows = min(TG_ROWS, n - r0);
        const bool more = r0 + TG_ROWS < n;
        if (more) {
            fetch(r0 + TG_ROWS);
        }
        for (int rr = 0; rr < rows; ++rr) {
            acc = fma(sBo[h][rr][kk], sV[h][rr][jj], acc);
        }
        if (more) {
            put(h ^ 1);
        }
        __syncthreads();
    }
    if (k0 + kk < m && j0 + jj < P) {
        T[(size_t)(j0 + jj) * m + k0 + kk] = acc;
    }
}

// Column chains: warp 0 of a block runs 32 column chains (lane = column) out
// of shared memory while warps 1..3 stage the next tile of rows.
constexpr int CC_COLS = 32, CC_ROWS = 64, CC_THREADS = 128;

// Fused chains over the rows i = 0..n-1 in order: the reference's sequential
// f64 accumulations (kernels.cc:361-366 norm of the stored column;
// kernels.cc:215-237 dot_widen; marsalgo.cc:359-369 column norms of X).
struct SqChain {  // sum of squares of the stored f32 column Bx[:, col[j]]
    static constexpr bool kUsesY = false;
    const float *Bx;
    size_t ld;
    const int *col;
    __device__ __forceinline__ float param(int) const { return 0.f; }
    __device__ __forceinline__ float load(size_t i, int j, float) const
    {
        return Bx[i + (size_t)(col ? col[j] : j) * ld];
    }
    __device__ __forceinline__ float yload(size_t) const { return 0.f; }
    __device__ __forceinline__ double step(double acc, double v, double) const
    {
        return fma(v, v, acc);
    }
    __device__ __forceinline__ double finish(double acc, int) const { return acc; }
};

template <class Op>
__global__ void __launch_bounds__(CC_THREADS) k_colchain(Op op, int n, int P, double *__restrict__ out)
{
    __shared__ double tile[2][CC_COLS][CC_ROWS + 1];
    __shared__ double ytile[2][CC_ROWS];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int j0 = blockIdx.x * CC_COLS;
    const int ncols = min(CC_COLS, P - j0);
    const int ntiles = (n + CC_ROWS - 1) / CC_ROWS;
    __shared__ float cparam[CC_COLS];
    if (t < ncols) {
        cparam[t] = op.param(j0 + t);
    }
    __syncthreads();
    auto load = [&](int tl, int b) {
        const int base = tl * CC_ROWS, rows = min(CC_ROWS, n - base);
        for (int e = t - 32; e < ncols * CC_ROWS; e += CC_THREADS - 32) {
            const int c = e / CC_ROWS, r = e % CC_ROWS;
            if (r < rows) {
                tile[b][c][r] = (double)op.load((size_t)(base + r), j0 + c, cparam[c]);
            }
        }
        if (Op::kUsesY) {
            for (int r = t - 32; r < rows; r += CC_THREADS - 32) {
                ytile[b][r] = (double)op.yload((size_t)(base + r));
            }
        }
    };
    if (warp > 0) {
        load(0, 0);
    }
    __syncthreads();
    double acc = 0.0;
    for (int tl = 0; tl < ntiles; ++tl) {
        const int b = tl & 1;
        if (warp == 0) {
            if (lane < ncols) {
                const int rows = min(CC_ROWS, n - tl * CC_ROWS);
                for (int r = 0; r < rows; ++r) {
                    acc = op.step(acc, tile[b][lane][r], ytile[b][r]);
                }
            }
        } else if (tl + 1 < ntiles) {
            load(tl + 1, b ^ 1);
        }
        __syncthreads();
    }
    if (warp == 0 && lane < ncols) {
        out[j0 + lane] = op.finish(acc, j0 + lane);
    }
}


// ---------------------------------------------------------------------------
// Bx <- f32(Bx - Bo T), one element per thread; the projection is the
// reference's fused chain over k from 0 (kernels.cc:56-118 scalar branches).
// ---------------------------------------------------------------------------
constexpr int PJ_THREADS = 128, PJ_COLS = 8;

template <class Src>
__global__ void __launch_bounds__(PJ_THREADS)
    k_project(Src src, const float *__restrict__ Bo, size_t ldbo, int n, int m, int P,
              const double *__restrict__ T, const int *__restrict__ out_col,
              float *__restrict__ Bx, size_t ldBx)
{
    extern __shared__ double sT[];  // PJ_COLS * m
    const int t = threadIdx.x, j0 = blockIdx.y * PJ_COLS;
    for (int e = t; e < PJ_COLS * m; e += PJ_THREADS) {
        const int q = e / m, k = e % m, j = j0 + q;
        sT[e] = (j < P) ? T[(size_t)j * m + k] : 0.0;
    }
    __syncthreads();
    const size_t i = (size_t)blockIdx.x * PJ_THREADS + t;
    if (i >= (size_t)n) {
        return;
    }
    const float *bo = Bo + i * ldbo;
    double proj[PJ_COLS];
#pragma unroll
    for (int q = 0; q < PJ_COLS; ++q) {
        proj[q] = 0.0;
    }
    // each column's chain runs over k in order; the conversion of bo[k] is shared
    for (int k = 0; k < m; ++k) {
        const double bk = (double)bo[k];
#pragma unroll
        for (int q = 0; q < PJ_COLS; ++q) {
            proj[q] = fma(bk, sT[q * m + k], proj[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < PJ_COLS; ++q) {
        const int j = j0 + q;
        if (j < P) {
            const double v = (double)src(i, j) - proj[q];
            const int oc = out_col ? out_col[j] : j;
            Bx[i + (size_t)oc * ldBx] = (float)v;
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

__device__ __forceinline__ float norm_scale(double s, double tol)
{
    return (s > tol) ? (float)(1.0 / sqrt(s + tol)) : 0.0f;
}

// ybx[j] = fused chain over i of f32(Bx[i,j] * scale_j) * y[i] (dot_widen of the
// normalised column, kernels.cc:215-237 after kernels.cc:401-416). The scale
// is applied when the tile is loaded.
struct NormDotChain {
    static constexpr bool kUsesY = true;
    const float *Bx;
    size_t ld;
    const float *y;
    const double *s;
    double tol;
    __device__ __forceinline__ float param(int j) const { return norm_scale(s[j], tol); }
    __device__ __forceinline__ float load(size_t i, int j, float scale) const
    {
        return Bx[i + (size_t)j * ld] * scale;
    }
    __device__ __forceinline__ float yload(size_t i) const { return y[i]; }
    __device__ __forceinline__ double step(double acc, double v, double yv) const
    {
        return fma(v, yv, acc);
    }
    __device__ __forceinline__ double finish(double acc, int) const { return acc; }
};

constexpr int NM_THREADS = 256, NM_COLS = 8;

__global__ void __launch_bounds__(NM_THREADS)
    k_scale(float *__restrict__ Bx, size_t ldBx, int n, int P, const double *__restrict__ s,
            double tol)
{
    __shared__ float sc[NM_COLS];
    const int t = threadIdx.x, j0 = blockIdx.y * NM_COLS;
    if (t < NM_COLS) {
        const int j = j0 + t;
        sc[t] = j < P ? norm_scale(s[j], tol) : 0.0f;
    }
    __syncthreads();
    const size_t i = (size_t)blockIdx.x * NM_THREADS + t;
    if (i >= (size_t)n) {
        return;
    }
    for (int q = 0; q < NM_COLS && j0 + q < P; ++q) {
        Bx[i + (size_t)(j0 + q) * ldBx] *= sc[q];
    }
}

// ---------------------------------------------------------------------------
// FP64 hinge sweep (marsalgo.cc:576-649 with covariates_impl :91-151), in the
// reference's operation order.
//
// Block = one input column and up to W candidates (parent columns):
//   warps 0..W-1  one candidate each; lane l holds components c = l + 32 q of
//                 the running f and g (component m is the candidate column Bx)
//   warp  W       the six scalar recurrences (k0, k1, w, bd, b2, vb) of all W
//                 candidates, one lane per candidate
//   warp  W+1     the loader: stages the next SW_ROWS sorted rows as doubles
//                 (permutation, delta, delta^2, y, the gathered Bo rows, B and
//                 Bx of every candidate) into the other half of a double buffer
// At a grid row each candidate warp saves f in a snapshot slot and the scalar
// warp saves k0 + k1 and w; when SW_SNAP slots are in use, lane q of each
// candidate warp scores slot q with the reference's sequential chains
// ff = sum_c f_c^2 and fy = sum_c f_c yc_c (c = 0..m) and the warp keeps the
// first maximum in row order.
// ---------------------------------------------------------------------------
constexpr int SW_ROWS = 32, SW_SNAP = 32, SW_MAXW = 8;

struct SweepSmem {
    // offsets (in doubles) into the dynamic shared memory
    size_t snap, bo, bd, bx, d, dd, yd, ybo, mk, mw, total;
    __host__ __device__ SweepSmem(int m, int W)
    {
        size_t o = 0;
        snap = o;
        o += (size_t)W * SW_SNAP * (m + 1);
        bo = o;
        o += 2 * (size_t)SW_ROWS * m;
        bd = o;
        o += 2 * (size_t)W * SW_ROWS;
        bx = o;
        o += 2 * (size_t)W * SW_ROWS;
        d = o;
        o += 2 * SW_ROWS;
        dd = o;
        o += 2 * SW_ROWS;
        yd = o;
        o += 2 * SW_ROWS;
        ybo = o;
        o += (size_t)m + 1;
        mk = o;
        o += (size_t)W * SW_SNAP;
        mw = o;
        o += (size_t)W * SW_SNAP;
        total = o;
    }
};

template <int CPL>
__global__ void __launch_bounds__(32 * (SW_MAXW + 2))
    k_sweep(const SweepTask *__restrict__ tasks, const int *__restrict__ perm,
            const float *__restrict__ xsort, const float *__restrict__ y,
            const float *__restrict__ B, size_t ldB, const int *__restrict__ cand_b,
            const float *__restrict__ Bx, size_t ldBx, const float *__restrict__ Bo,
            size_t ldbo, const double *__restrict__ ybo, const double *__restrict__ ybx, int n,
            int m, int head, int tail, int min_span, double tol, double *__restrict__ hsse,
            int *__restrict__ hrow)
{
    extern __shared__ double dyn[];
    const int W = (blockDim.x >> 5) - 2;  // candidate warps
    const SweepSmem L(m, W);
    const int ldF = m + 1;
    __shared__ int srow[SW_SNAP];

    const SweepTask task = tasks[blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool cwarp = warp < task.count;
    const bool swarp = warp == W;
    const bool lwarp = warp == W + 1;
    const int *pk = perm + (size_t)task.xcol * n;
    const float *xs = xsort + (size_t)task.xcol * n;

    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        dyn[L.ybo + c] = ybo[c];
    }
    // The loader stages rows [i0, i0 + rows) into buffer half h.
    auto stage = [&](int i0, int h) {
        const int rows = min(SW_ROWS, tail - i0);
        int k = 0;
        if (lane < rows) {
            const int i = i0 + lane;
            k = pk[i];
            dyn[L.yd + h * SW_ROWS + lane] = (double)y[k];
            const double d = i > 0 ? (double)(xs[i - 1] - xs[i]) : 0.0;
            dyn[L.d + h * SW_ROWS + lane] = d;
            dyn[L.dd + h * SW_ROWS + lane] = d * d;
            const float *row = Bo + (size_t)k * ldbo;
            double *dst = dyn + L.bo + ((size_t)h * SW_ROWS + lane) * m;
            for (int c = 0; c < m; ++c) {
                dst[c] = (double)row[c];
            }
            for (int cw = 0; cw < task.count; ++cw) {
                const int cand = task.cand0 + cw;
                dyn[L.bd + (h * W + cw) * SW_ROWS + lane] =
                    (double)B[(size_t)k + (size_t)cand_b[cand] * ldB];
                dyn[L.bx + (h * W + cw) * SW_ROWS + lane] =
                    (double)Bx[(size_t)k + (size_t)cand * ldBx];
            }
        }
    };

    const int mycand = task.cand0 + (cwarp ? warp : 0);
    const double ybx_c = ybx[mycand];
    double *snap = dyn + L.snap + (size_t)(cwarp ? warp : 0) * SW_SNAP * ldF;
    double *mk = dyn + L.mk, *mw = dyn + L.mw;
    double f[CPL], g[CPL];
#pragma unroll
    for (int q = 0; q < CPL; ++q) {
        f[q] = 0.0;
        g[q] = 0.0;
    }
    const bool slane = swarp && lane < task.count;
    double k0 = 0, k1 = 0, w = 0, bd = 0, vb = 0, b2 = 0;
    double best = 0.0;
    int besti = -1;
    int nsnap = 0;  // block-uniform
    long next_grid = (long)head + 1;

    auto flush = [&]() {
        if (cwarp) {
            double sse = -1.0;
            int row = 0x7fffffff;
            if (lane < nsnap) {
                const double *fs = snap + (size_t)lane * ldF;
                const double *yb = dyn + L.ybo;
                double ff = 0.0, fy = 0.0;
                for (int c = 0; c < m; ++c) {
                    ff = fma(fs[c], fs[c], ff);
                    fy = fma(fs[c], yb[c], fy);
                }
                ff = fma(fs[m], fs[m], ff);
                fy = fma(fs[m], ybx_c, fy);
                const double uw = fy - mw[warp * SW_SNAP + lane];
                const double den = mk[warp * SW_SNAP + lane] - ff;
                sse = den > tol ? (uw * uw) / (den + tol) : 0.0;
                row = srow[lane];
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
    };

    if (lwarp && tail > 0) {
        stage(0, 0);
    }
    __syncthreads();
    int h = 0;
    for (int i0 = 0; i0 < tail; i0 += SW_ROWS, h ^= 1) {
        const int rows = min(SW_ROWS, tail - i0);
        int gcount = 0;
        for (long gr = next_grid; gr < i0 + rows; gr += min_span) {
            ++gcount;
        }
        if (nsnap + gcount > SW_SNAP) {
            flush();
            __syncthreads();  // slots are rewritten below
        }
        if (cwarp) {
            const double *bw = dyn + L.bd + (h * W + warp) * SW_ROWS;
            const double *xw = dyn + L.bx + (h * W + warp) * SW_ROWS;
            const double *sd = dyn + L.d + h * SW_ROWS;
            const double *rowb = dyn + L.bo + (size_t)h * SW_ROWS * m;
            long ng = next_grid;
            int slot = nsnap;
            for (int r = 0; r < rows; ++r) {
                const int i = i0 + r;
                const double bk = bw[r], bxk = xw[r];
                const double *rowp = rowb + r * m;
                const double di = sd[r];  // 0 for the first row
#pragma unroll
                for (int q = 0; q < CPL; ++q) {
                    const int c = lane + 32 * q;
                    const double xv = c < m ? rowp[c] : (c == m ? bxk : 0.0);
                    f[q] = fma(di, g[q], f[q]);
                    g[q] = fma(bk, xv, g[q]);
                }
                if (i == ng) {
                    ng += min_span;
                    double *fs = snap + (size_t)slot * ldF;
#pragma unroll
                    for (int q = 0; q < CPL; ++q) {
                        const int c = lane + 32 * q;
                        if (c <= m) {
                            fs[c] = f[q];
                        }
                    }
                    if (lane == 0 && warp == 0) {
                        srow[slot] = i;
                    }
                    ++slot;
                }
            }
        } else if (slane) {
            const double *bw = dyn + L.bd + (h * W + lane) * SW_ROWS;
            const double *sd = dyn + L.d + h * SW_ROWS;
            const double *sdd = dyn + L.dd + h * SW_ROWS;
            const double *syd = dyn + L.yd + h * SW_ROWS;
            long ng = next_grid;
            int slot = nsnap;
            for (int r = 0; r < rows; ++r) {
                const int i = i0 + r;
                const double bk = bw[r], yk = syd[r];
                if (i == 0) {
                    vb = bk * yk;
                    b2 = bk * bk;
                    continue;
                }
                const double di = sd[r];
                k0 = fma(sdd[r], b2, k0);
                k1 = fma(di * 2, bd, k1);
                w = fma(di, vb, w);
                bd = fma(di, b2, bd);
                b2 = fma(bk, bk, b2);
                vb = fma(yk, bk, vb);
                if (i == ng) {
                    ng += min_span;
                    mk[lane * SW_SNAP + slot] = k0 + k1;
                    mw[lane * SW_SNAP + slot] = w;
                    ++slot;
                }
            }
        } else if (lwarp && i0 + SW_ROWS < tail) {
            stage(i0 + SW_ROWS, h ^ 1);
        }
        nsnap += gcount;
        next_grid += (long)gcount * min_span;
        __syncthreads();
    }
    if (nsnap > 0) {
        flush();
    }
    if (cwarp && lane == 0) {
        hsse[mycand] = best;
        hrow[mycand] = besti >= 0 ? pk[besti] : -1;
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


// ---------------------------------------------------------------------------
// Serial chains of the append, in the reference's row order
// (kernels.cc:194-281, marsalgo.cc:829-861). One block: thread 0 runs the
// fused-multiply-add chain out of shared memory while the other threads stage
// the next chunk of rows and write the previous chunk's updated v back.
// ---------------------------------------------------------------------------
constexpr int SER_THREADS = 256, SER_CH = 1024;

// Modified Gram-Schmidt pass j = 0..m: v <- v - c_{j-1} Bo[:, j-1] (fused),
// then c_j = sum_i Bo[i,j] v[i] (j < m) or ||v||^2 (j == m), rows in order.
// Leaves c_j in coef, sum_j c_j^2 in scal[0] and ||v||^2 in scal[1].
__global__ void __launch_bounds__(SER_THREADS)
    k_mgs_serial(const float *__restrict__ BoC, int n, int m, double *__restrict__ v,
                 double *__restrict__ coef, double *__restrict__ scal)
{
    __shared__ double sv[2][SER_CH];
    __shared__ float sp[2][SER_CH], sc[2][SER_CH];
    __shared__ double s_coef;
    const int t = threadIdx.x;
    const int nch = (n + SER_CH - 1) / SER_CH;
    double proj = 0.0;
    for (int j = 0; j <= m; ++j) {
        const float *prev = BoC + (size_t)(j > 0 ? j - 1 : 0) * n;
        const float *cur = BoC + (size_t)(j < m ? j : 0) * n;
        const double cprev = (j > 0) ? s_coef : 0.0;
        auto load = [&](int ch, int b) {
            const int base = ch * SER_CH, cnt = min(SER_CH, n - base);
            for (int e = t - 1; e < cnt; e += SER_THREADS - 1) {
                sv[b][e] = v[base + e];
                sp[b][e] = prev[base + e];
                sc[b][e] = cur[base + e];
            }
        };
        auto store = [&](int ch, int b) {
            const int base = ch * SER_CH, cnt = min(SER_CH, n - base);
            for (int e = t - 1; e < cnt; e += SER_THREADS - 1) {
                v[base + e] = sv[b][e];
            }
        };
        if (t > 0) {
            load(0, 0);
        }
        __syncthreads();
        double acc = 0.0;
        for (int ch = 0; ch < nch; ++ch) {
            const int b = ch & 1;
            if (t == 0) {
                const int cnt = min(SER_CH, n - ch * SER_CH);
                for (int e = 0; e < cnt; ++e) {
                    double vi = sv[b][e];
                    if (j > 0) {
                        vi = fma(-cprev, (double)sp[b][e], vi);
                        sv[b][e] = vi;
                    }
                    acc = (j < m) ? fma((double)sc[b][e], vi, acc) : fma(vi, vi, acc);
                }
            } else {
                if (ch > 0 && j > 0) {
                    store(ch - 1, b ^ 1);
                }
                if (ch + 1 < nch) {
                    load(ch + 1, b ^ 1);
                }
            }
            __syncthreads();
        }
        if (t > 0 && j > 0) {
            store(nch - 1, (nch - 1) & 1);
        }
        if (t == 0) {
            if (j < m) {
                coef[j] = acc;
                s_coef = acc;
                proj = fma(acc, acc, proj);
            } else {
                scal[0] = proj;
                scal[1] = acc;
            }
        }
        __syncthreads();
    }
}

// out = sum_i a_i b_i as one fused chain over the rows in order.
struct VSq {  // (v, v)
    const double *v;
    __device__ __forceinline__ void operator()(int i, double &a, double &b) const
    {
        a = v[i];
        b = v[i];
    }
};
struct ColDotY {  // ((double)Q[i], (double)y[i])
    const float *q;
    const float *y;
    __device__ __forceinline__ void operator()(int i, double &a, double &b) const
    {
        a = (double)q[i];
        b = (double)y[i];
    }
};

template <class Op>
__global__ void __launch_bounds__(SER_THREADS)
    k_serial_dot(Op op, int n, double *__restrict__ out)
{
    __shared__ double sa[2][SER_CH], sb[2][SER_CH];
    const int t = threadIdx.x;
    const int nch = (n + SER_CH - 1) / SER_CH;
    auto load = [&](int ch, int b) {
        const int base = ch * SER_CH, cnt = min(SER_CH, n - base);
        for (int e = t - 1; e < cnt; e += SER_THREADS - 1) {
            op(base + e, sa[b][e], sb[b][e]);
        }
    };
    if (t > 0) {
        load(0, 0);
    }
    __syncthreads();
    double acc = 0.0;
    for (int ch = 0; ch < nch; ++ch) {
        const int b = ch & 1;
        if (t == 0) {
            const int cnt = min(SER_CH, n - ch * SER_CH);
            for (int e = 0; e < cnt; ++e) {
                acc = fma(sa[b][e], sb[b][e], acc);
            }
        } else if (ch + 1 < nch) {
            load(ch + 1, b ^ 1);
        }
        __syncthreads();
    }
    if (t == 0) {
        *out = acc;
    }
}

__global__ void __launch_bounds__(AP_THREADS)
    k_append_fill(char type, const float *__restrict__ X, size_t ldX, const float *__restrict__ s,
                  int xcol, float *__restrict__ B, size_t ldB, int bcol, int m, float h, int n,
                  double *__restrict__ v)
{
    const float sx = s[xcol];
    for (int i = blockIdx.x * AP_THREADS + threadIdx.x; i < n; i += gridDim.x * AP_THREADS) {
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
        v[i] = (double)val;
    }
}

// B[:, m] /= f32(sqrt(raw2)) (marsalgo.cc:829-836).
__global__ void __launch_bounds__(AP_THREADS)
    k_append_scale(float *__restrict__ B, size_t ldB, int m, int n, const double *__restrict__ raw2)
{
    const float raw = (float)sqrt(*raw2);
    for (int i = blockIdx.x * AP_THREADS + threadIdx.x; i < n; i += gridDim.x * AP_THREADS) {
        B[(size_t)i + (size_t)m * ldB] /= raw;
    }
}

// v /= w; column m of Bo (row-major) and BoC = f32(v) (kernels.cc:274-279,
// marsalgo.cc:846-850).
__global__ void __launch_bounds__(AP_THREADS)
    k_append_store(double w, double *__restrict__ v, float *__restrict__ Bo, size_t ldbo,
                   float *__restrict__ BoC, int n, int m)
{
    for (int i = blockIdx.x * AP_THREADS + threadIdx.x; i < n; i += gridDim.x * AP_THREADS) {
        const double vi = v[i] / w;
        v[i] = vi;
        const float vf = (float)vi;
        Bo[(size_t)i * ldbo + m] = vf;
        BoC[(size_t)m * n + i] = vf;
    }
}


}  // namespace

int append_blocks(int n) { return (int)std::max<size_t>(1, std::min<size_t>(608, ceil_div(n, 2048))); }

template <class Src>
void tgemm_fp64(cudaStream_t st, const Src &src, const float *Bo, size_t ldbo, int n, int m,
                int P, double *T, long long *launches)
{
    if (P <= 0 || m <= 0) {
        return;
    }
    int kt = 4;  // narrower tiles would need more than 48 KB of static shared memory
    while (kt < m && kt < 32) {
        kt *= 2;
    }
    const unsigned gx = (unsigned)ceil_div(m, kt), gy = (unsigned)ceil_div(P, TG_THREADS / kt);
    verify(gy <= 65535, "too many candidate columns for one launch", 2);
#define TG_CASE(K)                                                                    \
    case K:                                                                           \
        k_tgemm<Src, K><<<dim3(gx, gy), TG_THREADS, 0, st>>>(src, Bo, ldbo, n, m, P, T); \
        break;
    switch (kt) {
        TG_CASE(4)
        TG_CASE(8)
        TG_CASE(16)
        TG_CASE(32)
    }
#undef TG_CASE
    LAUNCH_CHECK();
    *launches += 1;
}

template void tgemm_fp64<FillSrc>(cudaStream_t, const FillSrc &, const float *, size_t, int, int,
                                  int, double *, long long *);
template void tgemm_fp64<StoredSrc>(cudaStream_t, const StoredSrc &, const float *, size_t, int,
                                    int, int, double *, long long *);

template <class Op>
void colchain(cudaStream_t st, const Op &op, int n, int P, double *out, long long *launches)
{
    if (P <= 0) {
        return;
    }
    k_colchain<Op><<<(unsigned)ceil_div(P, CC_COLS), CC_THREADS, 0, st>>>(op, n, P, out);
    LAUNCH_CHECK();
    *launches += 1;
}

template <class Src>
void project_fp64(cudaStream_t st, const Src &src, const float *Bo, size_t ldbo, int n, int m,
                  int P, const int *out_col, float *Bx, size_t ldBx, double *s_out,
                  const ProjectScratch &ws, long long *launches)
{
    if (P <= 0) {
        return;
    }
    tgemm_fp64(st, src, Bo, ldbo, n, m, P, ws.T, launches);
    const int rb = (int)ceil_div(n, PJ_THREADS);
    const size_t smem = sizeof(double) * PJ_COLS * std::max(m, 1);
    if (smem > 48 * 1024) {
        CUDA_CHECK(cudaFuncSetAttribute(k_project<Src>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
    }
    verify(ceil_div(P, PJ_COLS) <= 65535, "too many candidate columns for one launch", 2);
    k_project<Src><<<dim3(rb, (unsigned)ceil_div(P, PJ_COLS)), PJ_THREADS, smem, st>>>(
        src, Bo, ldbo, n, m, P, ws.T, out_col, Bx, ldBx);
    LAUNCH_CHECK();
    *launches += 1;
    colchain(st, SqChain{Bx, ldBx, out_col}, n, P, s_out, launches);
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
                   double tol, const float *y, bool store, double *ybx, long long *launches)
{
    if (P <= 0) {
        return;
    }
    colchain(st, NormDotChain{Bx, ldBx, y, s, tol}, n, P, ybx, launches);
    if (store) {
        verify(ceil_div(P, NM_COLS) <= 65535, "too many candidate columns for one launch", 2);
        k_scale<<<dim3((unsigned)ceil_div(n, NM_THREADS), (unsigned)ceil_div(P, NM_COLS)),
                  NM_THREADS, 0, st>>>(Bx, ldBx, n, P, s, tol);
        LAUNCH_CHECK();
        *launches += 1;
    }
}

void scale_columns(cudaStream_t st, float *Bx, size_t ldBx, int n, int P, const double *s,
                   double tol, long long *launches)
{
    if (P <= 0) {
        return;
    }
    verify(ceil_div(P, NM_COLS) <= 65535, "too many candidate columns for one launch", 2);
    k_scale<<<dim3((unsigned)ceil_div(n, NM_THREADS), (unsigned)ceil_div(P, NM_COLS)), NM_THREADS,
              0, st>>>(Bx, ldBx, n, P, s, tol);
    LAUNCH_CHECK();
    *launches += 1;
}

// Candidate warps per sweep block: at most 4, fewer when the launch has few
// candidates (two blocks per SM) or the snapshots would not fit.
static size_t sweep_smem(int m, int w) { return sizeof(double) * SweepSmem(m, w).total; }

int sweep_warps(int m, int candidates)
{
    int w = 4;
    while (w > 2 && (candidates + w - 1) / w < 2 * 152) {
        --w;
    }
    while (w > 1 && sweep_smem(m, w) > 200 * 1024) {
        --w;
    }
    return w;
}

void sweep_fp64(cudaStream_t st, const SweepTask *tasks, int ntasks, const int *perm,
                const float *xsort, const float *y, const float *B, size_t ldB,
                const int *cand_b, const float *Bx, size_t ldBx, const float *Bo, size_t ldbo,
                const double *ybo, const double *ybx, int n, int m, int head, int tail,
                int min_span, double tol, double *hsse, int *hrow, int warps_per_block,
                long long *launches)
{
    if (ntasks <= 0) {
        return;
    }
    const int warps = warps_per_block;
    const size_t smem = sweep_smem(m, warps);
    verify(smem <= 227 * 1024, "the GPU hinge sweep supports at most 430 basis functions");
    const int comps = m + 1;
#define LAUNCH_SWEEP(CPL)                                                                      \
    do {                                                                                       \
        CUDA_CHECK(cudaFuncSetAttribute(k_sweep<CPL>,                                          \
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,           \
                                        (int)smem));                                           \
        k_sweep<CPL><<<ntasks, 32 * (warps + 2), smem, st>>>(                                  \
            tasks, perm, xsort, y, B, ldB, cand_b, Bx, ldBx, Bo, ldbo, ybo, ybx, n, m, head,   \
            tail, min_span, tol, hsse, hrow);                                                  \
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
        *launches += 2;  // the radix sort's own kernels are not counted
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
    const int nb = append_blocks(n);
    k_append_fill<<<nb, AP_THREADS, 0, st>>>(type, X, ldX, s, xcol, B, ldB, bcol, m, h, n, ws.v);
    LAUNCH_CHECK();
    k_serial_dot<VSq><<<1, SER_THREADS, 0, st>>>(VSq{ws.v}, n, ws.scal + 3);
    LAUNCH_CHECK();
    k_append_scale<<<nb, AP_THREADS, 0, st>>>(B, ldB, m, n, ws.scal + 3);
    LAUNCH_CHECK();
    *launches += 3;
}

void mgs_pass(cudaStream_t st, const float *BoC, int n, int m, const AppendScratch &ws,
              long long *launches)
{
    k_mgs_serial<<<1, SER_THREADS, 0, st>>>(BoC, n, m, ws.v, ws.coef, ws.scal);
    LAUNCH_CHECK();
    *launches += 1;
}

void append_store(cudaStream_t st, double w, float *Bo, size_t ldbo, float *BoC, int n, int m,
                  const float *y, const AppendScratch &ws, long long *launches)
{
    k_append_store<<<append_blocks(n), AP_THREADS, 0, st>>>(w, ws.v, Bo, ldbo, BoC, n, m);
    LAUNCH_CHECK();
    k_serial_dot<ColDotY><<<1, SER_THREADS, 0, st>>>(ColDotY{BoC + (size_t)m * n, y}, n,
                                                     ws.scal + 2);
    LAUNCH_CHECK();
    *launches += 2;
}

// sum_i X[i,j]^2 per column as the reference's sequential fused chain
// (marsalgo.cc:359-369).
struct XSqChain {
    static constexpr bool kUsesY = false;
    const float *X;
    size_t ld;
    __device__ __forceinline__ float param(int) const { return 0.f; }
    __device__ __forceinline__ float load(size_t i, int j, float) const { return X[i + (size_t)j * ld]; }
    __device__ __forceinline__ float yload(size_t) const { return 0.f; }
    __device__ __forceinline__ double step(double acc, double v, double) const
    {
        return fma(v, v, acc);
    }
    __device__ __forceinline__ double finish(double acc, int) const { return acc; }
};

void column_sumsq(cudaStream_t st, const float *X, size_t ldX, int n, int p, double *out,
                  long long *launches)
{
    colchain(st, XSqChain{X, ldX}, n, p, out, launches);
}

}  // namespace mgpu
