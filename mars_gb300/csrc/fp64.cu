// FP64 forward-pass kernels (the plain FP64 GPU path; also the re-decision
// path of the mixed mode). Arithmetic follows the reference CPU path
// operation for operation where the order is local (per element, per
// candidate); long reductions over rows are split deterministically
// (fixed per-thread order, fixed block tree, fixed order across blocks).
#include "fp64.cuh"
#include "xchain.cuh"
#include "xhinge.cuh"

#include <type_traits>

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

namespace mgpu {
namespace {

// ---------------------------------------------------------------------------
// T = Bo^T Bx with every entry accumulated over the rows in order
// i = 0..n-1 by one fused-multiply-add chain, which is the reference's order
// (kernels.cc:327-335: tc[k] += bo_row[k] * bx[i], rows outermost). The block
// tile is KT components x (128 / KT) columns, one chain per thread.
//
// GB300's FP64 pipe issues one warp instruction per ~64 cycles per SM
// sub-partition, conversions to f64 included, and a lone dependent chain
// advances once per ~86 cycles. So every operand is converted to f64 exactly
// once, with all lanes busy, and the chains see only f64 loads and FMAs:
//   - rows arrive TG_ROWS at a time through a TG_STAGES-deep cp.async ring
//     (Bo as stored -- the device copy of the fit state is f64 -- and the raw
//     f32 candidate columns);
//   - in the iteration before a tile's chain steps, the block converts it:
//     the candidate value (for FillSrc the f32 product B * (X * s)) once per
//     element, and Bo when it is stored as f32;
//   - the chain steps of the tile before run meanwhile.
// ---------------------------------------------------------------------------
constexpr int TG_ROWS = 32, TG_THREADS = 128, TG_STAGES = 4;

__host__ __device__ constexpr size_t align16(size_t b) { return (b + 15) / 16 * 16; }

template <class BoT, int KT, int R>
struct TgemmSmem {
    static constexpr int JT = TG_THREADS / KT;
    static constexpr bool kConvBo = sizeof(BoT) != sizeof(double);
    static constexpr size_t rawBo = 0;  // [TG_STAGES][TG_ROWS][KT + 1] BoT
    static constexpr size_t rawV =      // [TG_STAGES][R][JT][TG_ROWS + 1] f32
        align16(rawBo + sizeof(BoT) * TG_STAGES * TG_ROWS * (KT + 1));
    static constexpr size_t dV =  // [2][JT][TG_ROWS + 1] f64
        align16(rawV + 4 * TG_STAGES * R * JT * (TG_ROWS + 1));
    static constexpr size_t dBo =  // [2][TG_ROWS][KT + 1] f64 (f32 Bo only)
        align16(dV + 8 * 2 * JT * (TG_ROWS + 1));
    static constexpr size_t total = align16(dBo + (kConvBo ? 8 * 2 * TG_ROWS * (KT + 1) : 0));
};

template <class Src, class BoT, int KT>
__global__ void __launch_bounds__(TG_THREADS)
    k_tgemm(Src src, const BoT *__restrict__ Bo, size_t ldbo, int n, int m, int P,
            double *__restrict__ T)
{
    constexpr int R = Src::kRaw, S = TG_STAGES;
    using L = TgemmSmem<BoT, KT, R>;
    constexpr int JT = L::JT;
    extern __shared__ __align__(16) unsigned char tsm[];
    auto rBo = reinterpret_cast<BoT(*)[TG_ROWS][KT + 1]>(tsm + L::rawBo);
    auto rV = reinterpret_cast<float(*)[R][JT][TG_ROWS + 1]>(tsm + L::rawV);
    auto dV = reinterpret_cast<double(*)[JT][TG_ROWS + 1]>(tsm + L::dV);
    auto dBo = reinterpret_cast<double(*)[TG_ROWS][KT + 1]>(tsm + L::dBo);
    __shared__ const float *vcol[R][JT];
    __shared__ float vprm[JT];
    const int t = threadIdx.x, kk = t % KT, jj = t / KT;
    const int k0 = blockIdx.x * KT, j0 = blockIdx.y * JT;
    if (t < JT) {
        const int j = j0 + t;
        vcol[0][t] = j < P ? src.raw0(j) : nullptr;
        vcol[R - 1][t] = j < P ? src.raw1(j) : nullptr;
        vprm[t] = j < P ? src.param(j) : 0.f;
    }
    __syncthreads();
    const int ntiles = (n + TG_ROWS - 1) / TG_ROWS;
    auto issue = [&](int tl) {
        const int sg = tl % S, r0 = tl * TG_ROWS;
        for (int e = t; e < TG_ROWS * KT; e += TG_THREADS) {
            const int rr = e / KT, cc = e % KT;
            const bool ok = r0 + rr < n && k0 + cc < m;
            cp_async<sizeof(BoT)>(&rBo[sg][rr][cc],
                                  ok ? Bo + (size_t)(r0 + rr) * ldbo + k0 + cc : Bo, ok);
        }
        for (int e = t; e < R * JT * TG_ROWS; e += TG_THREADS) {
            const int rr = e % TG_ROWS, cj = (e / TG_ROWS) % JT, q = e / (TG_ROWS * JT);
            const float *col = vcol[q][cj];
            const bool ok = col != nullptr && r0 + rr < n;
            cp_async4(&rV[sg][q][cj][rr], ok ? col + r0 + rr : vcol[0][0], ok);
        }
    };
    auto convert = [&](int tl) {  // raw tile tl (landed) -> f64 slot tl & 1
        const int sg = tl % S, h = tl & 1;
        for (int e = t; e < JT * TG_ROWS; e += TG_THREADS) {
            const int cj = e / TG_ROWS, rr = e % TG_ROWS;
            dV[h][cj][rr] = (double)src.combine(rV[sg][0][cj][rr], rV[sg][R - 1][cj][rr], vprm[cj]);
        }
        if (L::kConvBo) {
            for (int e = t; e < TG_ROWS * KT; e += TG_THREADS) {
                const int rr = e / KT, cc = e % KT;
                dBo[h][rr][cc] = (double)rBo[sg][rr][cc];
            }
        }
    };
#pragma unroll
    for (int q = 0; q < S - 1; ++q) {
        if (q < ntiles) {
            issue(q);
        }
        cp_async_commit();
    }
    cp_async_wait<S - 3>();  // tiles 0 and 1 landed
    __syncthreads();
    if (ntiles > 0) {
        convert(0);
    }
    __syncthreads();
    double acc = 0.0;
    for (int tl = 0; tl < ntiles; ++tl) {
        const int h = tl & 1;
        if (tl + S - 1 < ntiles) {
            issue(tl + S - 1);  // into the ring slot of tile tl - 1 (converted and consumed)
        }
        cp_async_commit();
        if (tl + 1 < ntiles) {
            convert(tl + 1);
        }
        const double *bo = L::kConvBo ? &dBo[h][0][kk]
                                      : reinterpret_cast<const double *>(&rBo[tl % S][0][kk]);
        const double *v = dV[h][jj];
        const int rows = min(TG_ROWS, n - tl * TG_ROWS);
        if (rows == TG_ROWS) {
#pragma unroll 8
            for (int rr = 0; rr < TG_ROWS; ++rr) {
                acc = fma(bo[rr * (KT + 1)], v[rr], acc);
            }
        } else {
            for (int rr = 0; rr < rows; ++rr) {
                acc = fma(bo[rr * (KT + 1)], v[rr], acc);
            }
        }
        cp_async_wait<S - 3>();  // tile tl + 2 landed
        __syncthreads();
    }
    if (k0 + kk < m && j0 + jj < P) {
        T[(size_t)(j0 + jj) * m + k0 + kk] = acc;
    }
}

// Column chains: warp 0 of a block runs 32 column chains (lane = column) in
// f64 out of shared memory. Warps 1..3 keep CC_STAGES - 1 tiles of raw f32
// rows in flight with cp.async (one warp instruction = 32 consecutive rows of
// one column) and convert the next tile to f64 once per element while warp 0
// steps through the current one.
constexpr int CC_COLS = 32, CC_ROWS = 32, CC_STAGES = 4, CC_THREADS = 128;

// Fused chains over the rows i = 0..n-1 in order: the reference's sequential
// f64 accumulations (kernels.cc:361-366 norm of the stored column;
// kernels.cc:215-237 dot_widen; marsalgo.cc:359-369 column norms of X).
// column(j) is the f32 column read by chain j, value() the f32 operand made
// from its raw value and param(j); step() runs on the f64 conversions.
struct SqChain {  // sum of squares of the stored f32 column Bx[:, col[j]]
    static constexpr bool kUsesY = false;
    const float *Bx;
    size_t ld;
    const int *col;
    __device__ __forceinline__ const float *column(int j) const
    {
        return Bx + (size_t)(col ? col[j] : j) * ld;
    }
    __device__ __forceinline__ const float *ycolumn() const { return nullptr; }
    __device__ __forceinline__ float param(int) const { return 0.f; }
    __device__ __forceinline__ float value(float v, float) const { return v; }
    __device__ __forceinline__ double step(double acc, double v, double) const
    {
        return fma(v, v, acc);
    }
};

template <class Op>
__global__ void __launch_bounds__(CC_THREADS) k_colchain(Op op, int n, int P, double *__restrict__ out)
{
    constexpr int LOADERS = CC_THREADS / 32 - 1, S = CC_STAGES;
    __shared__ float raw[S][CC_COLS][CC_ROWS + 1];
    __shared__ float yraw[S][CC_ROWS];
    __shared__ double dt[2][CC_COLS][CC_ROWS + 1];
    __shared__ double dy[2][CC_ROWS];
    __shared__ const float *cptr[CC_COLS];
    __shared__ float cparam[CC_COLS];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int j0 = blockIdx.x * CC_COLS;
    const int ncols = min(CC_COLS, P - j0);
    const int ntiles = (n + CC_ROWS - 1) / CC_ROWS;
    if (t < ncols) {
        cptr[t] = op.column(j0 + t);
        cparam[t] = op.param(j0 + t);
    }
    __syncthreads();
    const float *yc = op.ycolumn();
    const int lt = t - 32;  // loader thread index
    auto issue = [&](int tl) {
        const int sg = tl % S, i = tl * CC_ROWS + lane;
        const bool ok = i < n;
        for (int c = warp - 1; c < ncols; c += LOADERS) {
            cp_async4(&raw[sg][c][lane], cptr[c] + (ok ? i : 0), ok);
        }
        if (Op::kUsesY && warp == 1) {
            cp_async4(&yraw[sg][lane], yc + (ok ? i : 0), ok);
        }
    };
    auto convert = [&](int tl) {  // raw tile tl (landed) -> f64 slot tl & 1
        const int sg = tl % S, h = tl & 1;
        for (int e = lt; e < ncols * CC_ROWS; e += 32 * LOADERS) {
            const int c = e / CC_ROWS, r = e % CC_ROWS;
            dt[h][c][r] = (double)op.value(raw[sg][c][r], cparam[c]);
        }
        if (Op::kUsesY && lt < CC_ROWS) {
            dy[h][lt] = (double)yraw[sg][lt];
        }
    };
    if (warp > 0) {
#pragma unroll
        for (int q = 0; q < S - 1; ++q) {
            if (q < ntiles) {
                issue(q);
            }
            cp_async_commit();
        }
        cp_async_wait<S - 3>();  // tiles 0 and 1 landed
    }
    __syncthreads();
    if (warp > 0 && ntiles > 0) {
        convert(0);
    }
    __syncthreads();
    double acc = 0.0;
    for (int tl = 0; tl < ntiles; ++tl) {
        const int h = tl & 1;
        if (warp == 0) {
            if (lane < ncols) {
                const double *col = dt[h][lane];
                const double *yr = dy[h];
                const int rows = min(CC_ROWS, n - tl * CC_ROWS);
                if (rows == CC_ROWS) {
#pragma unroll 8
                    for (int r = 0; r < CC_ROWS; ++r) {
                        acc = op.step(acc, col[r], Op::kUsesY ? yr[r] : 0.0);
                    }
                } else {
                    for (int r = 0; r < rows; ++r) {
                        acc = op.step(acc, col[r], Op::kUsesY ? yr[r] : 0.0);
                    }
                }
            }
        } else {
            if (tl + S - 1 < ntiles) {
                issue(tl + S - 1);  // into the ring slot of tile tl - 1 (already converted)
            }
            cp_async_commit();
            if (tl + 1 < ntiles) {
                convert(tl + 1);
            }
            cp_async_wait<S - 3>();  // tile tl + 2 landed
        }
        __syncthreads();
    }
    if (warp == 0 && lane < ncols) {
        out[j0 + lane] = acc;
    }
}

// The same column chains, exact and parallel over the rows (xchain.cuh): one
// block per chain, one chunk of L consecutive rows per thread. Each thread sums
// its chunk in float-float; a block scan of those sums guesses every chunk's
// entry value; each thread runs its chunk XC_RUNS times from its guess (thread
// 0 runs chunk 0 once, from the true start 0); thread 0 then walks the chunks in
// order, translating a run's end or re-running the chunk. The value equals the
// chain k_colchain runs, bit for bit.
constexpr int XC_MAXK = 512;

// The terms of column chain j of a chain op (column(j) through value(), and
// ycolumn() or the value again).
template <class Op>
struct ColTerms {
    const float *col, *yc;
    float prm;
    Op op;
    __device__ __forceinline__ void operator()(int i, float &a, float &b) const
    {
        const float v = op.value(__ldg(col + i), prm);
        a = v;
        if constexpr (Op::kUsesY) {
            b = __ldg(yc + i);
        } else {
            b = v;
        }
    }
};
template <class Op>
struct ColChains {
    Op op;
    __device__ __forceinline__ ColTerms<Op> chain(int j) const
    {
        return {op.column(j), op.ycolumn(), op.param(j), op};
    }
};

template <class Chains>
__global__ void __launch_bounds__(XC_MAXK) k_xchain(Chains chains, int n, int L,
                                                    double *__restrict__ out)
{
    __shared__ XcChunk ch[XC_MAXK];
    __shared__ double wsum[XC_MAXK / 32];
    const int j = blockIdx.x, t = threadIdx.x, K = blockDim.x;
    const int lane = t & 31, warp = t >> 5, nw = K >> 5;
    const auto term = chains.chain(j);
    const int i0 = (int)min((long long)n, (long long)t * L), i1 = min(n, i0 + L);

    XcGuess g;
    for (int i = i0; i < i1; ++i) {
        float a, b;
        term(i, a, b);
        g.add_product(a, b);
    }
    const double v = g.value();
    double inc = v;  // inclusive prefix within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) {
            inc += u;
        }
    }
    if (lane == 31) {
        wsum[warp] = inc;
    }
    __syncthreads();
    if (warp == 0) {
        double w = lane < nw ? wsum[lane] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) {
                w += u;
            }
        }
        if (lane < nw) {
            wsum[lane] = w;
        }
    }
    __syncthreads();
    const double guess = (inc - v) + (warp > 0 ? wsum[warp - 1] : 0.0);
    double acc = 0.0;
    if (t == 0) {
        acc = xc_run(term, i0, i1, 0.0);
    } else {
        xc_speculate(term, i0, i1, guess, ch[t]);
    }
    __syncthreads();
    if (t == 0) {
        for (int c = 1; c < K; ++c) {
            const int c0 = (int)min((long long)n, (long long)c * L), c1 = min(n, c0 + L);
            bool redone = false;
            acc = xc_resolve(term, c0, c1, ch[c], acc, &redone);
        }
        out[j] = acc;
    }
}


// ---------------------------------------------------------------------------
// Bx <- f32(Bx - Bo T), one element per thread; the projection is the
// reference's fused chain over k from 0 (kernels.cc:56-118 scalar branches).
// ---------------------------------------------------------------------------
constexpr int PJ_THREADS = 128, PJ_COLS = 8;

template <class Src, class BoT>
__global__ void __launch_bounds__(PJ_THREADS)
    k_project(Src src, const BoT *__restrict__ Bo, size_t ldbo, int n, int m, int P,
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
    const BoT *bo = Bo + i * ldbo;
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
struct NormDotChain {  // ybx = sum_i f32(Bx[i, j] * scale_j) * y[i]
    static constexpr bool kUsesY = true;
    const float *Bx;
    size_t ld;
    const float *y;
    const double *s;
    double tol;
    __device__ __forceinline__ const float *column(int j) const { return Bx + (size_t)j * ld; }
    __device__ __forceinline__ const float *ycolumn() const { return y; }
    __device__ __forceinline__ float param(int j) const { return norm_scale(s[j], tol); }
    __device__ __forceinline__ float value(float v, float scale) const { return v * scale; }
    __device__ __forceinline__ double step(double acc, double v, double yv) const
    {
        return fma(v, yv, acc);
    }
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
//   warp  W       the loader: keeps S - 1 stages of SW_ROWS sorted rows in
//                 flight with cp.async -- each gathered row of the f64 Bo is
//                 one warp instruction (lanes over components); the B and Bx
//                 values of every candidate (f32, lanes over rows) are
//                 converted to f64 once, one stage ahead of their use; the
//                 deltas of the sorted x are formed at issue from the
//                 permutation and x prefetched one stage ahead
// The six scalar recurrences (k0, k1, w and their helpers) do not depend on
// the basis and come precomputed per grid row from k_hinge_scalars. At a grid
// row each candidate warp saves f in a snapshot slot; when SW_SNAP slots are
// in use, lane q of each candidate warp scores slot q with the reference's
// sequential chains ff = sum_c f_c^2 and fy = sum_c f_c yc_c (c = 0..m),
// den = (k0 + k1) - ff, uw = fy - w, and the warp keeps the first maximum in
// row order.
// ---------------------------------------------------------------------------
constexpr int SW_ROWS = 32, SW_SNAP = 32, SW_MAXW = 5;

struct SweepSmem {
    // byte offsets into the dynamic shared memory (f64 regions first)
    size_t snap, ybo, bo, cvt, raw, total;
    __host__ __device__ SweepSmem(int m, int W, int S)
    {
        size_t o = 0;
        snap = o;
        o += 8 * (size_t)W * SW_SNAP * (m + 1);
        ybo = o;
        o += 8 * ((size_t)m + 1);
        o = (o + 15) / 16 * 16;  // 16-byte cp.async destinations
        bo = o;  // [S][SW_ROWS][mp] f64 rows of Bo, row stride mp = m rounded up to 2
        o += 8 * (size_t)S * SW_ROWS * ((m + 1) / 2 * 2);
        cvt = o;  // [2][2W + 1][SW_ROWS] f64: B and Bx of each candidate, then the deltas
        o += 8 * 2 * (size_t)(2 * W + 1) * SW_ROWS;
        raw = o;  // [S][2W * SW_ROWS + SW_ROWS + 1] f32: B, Bx, then x from row i0 - 1
        o += 4 * (size_t)S * (2 * W * SW_ROWS + SW_ROWS + 1);
        total = (o + 15) / 16 * 16;
    }
};

template <int CPL, int S>
__global__ void __launch_bounds__(32 * (SW_MAXW + 1), 1)
    k_sweep(const SweepTask *__restrict__ tasks, const int *__restrict__ perm,
            const float *__restrict__ xsort, const float *__restrict__ bs,
            const float *__restrict__ bxs, const double *__restrict__ Bo, size_t ldbo,
            const double *__restrict__ ybo, const double *__restrict__ ybx,
            const double *__restrict__ scal, int ngrid, int n, int m, int head, int tail,
            int min_span, double tol, double *__restrict__ hsse, int *__restrict__ hrow,
            double *__restrict__ part, int split)
{
    extern __shared__ __align__(16) unsigned char sraw[];
    const int W = (blockDim.x >> 5) - 1;  // candidate warps
    const int NV = 2 * W + 1;
    const int RAW = 2 * W * SW_ROWS + SW_ROWS + 1;
    const int U = (m + 1) / 2, MP = 2 * U;  // 16-byte units per Bo row, padded row stride
    const SweepSmem L(m, W, S);
    const int ldF = m + 1;
    double *snapbase = reinterpret_cast<double *>(sraw + L.snap);
    double *sybo = reinterpret_cast<double *>(sraw + L.ybo);
    double *sbo = reinterpret_cast<double *>(sraw + L.bo);
    double *scvt = reinterpret_cast<double *>(sraw + L.cvt);  // [2][NV][SW_ROWS]
    float *sraw4 = reinterpret_cast<float *>(sraw + L.raw);   // [S][RAW]
    __shared__ int srow[SW_SNAP];

    const SweepTask task = tasks[blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // `split` warps share a candidate, each with its own components (lane +
    // 32 (sub + split q)): a candidate's FP64 FMAs per row are spread over as
    // many sub-partitions. Sub-warp 0 scores the cuts.
    const int wc = warp / split, sub = warp - wc * split;
    const bool cwarp = warp < task.count * split;
    const bool lwarp = warp == W;
    const int *pk = perm + (size_t)task.xcol * n;
    const float *xs = xsort + (size_t)task.xcol * n;
    const float *bsb = bs + (size_t)task.cand0 * n;
    const float *bxb = bxs + (size_t)task.cand0 * n;

    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        sybo[c] = ybo[c];
    }
    __syncthreads();

    const int nstages = (tail + SW_ROWS - 1) / SW_ROWS;
    // Loader: the permutation of this lane's row in the next stage to issue,
    // prefetched one stage ahead (it addresses the Bo row gathers).
    int pf_k = 0;
    auto prefetch = [&](int sq) {
        const int i = sq * SW_ROWS + lane;
        if (sq < nstages && i < tail) {
            pf_k = pk[i];
        }
    };
    auto issue = [&](int sq) {
        const int sg = sq % S, i0 = sq * SW_ROWS;
        const int rows = min(SW_ROWS, tail - i0);
        const int k = pf_k;
        double *bo = sbo + (size_t)sg * SW_ROWS * MP;
        // Bo rows, 16 bytes per lane, 32 / U rows per instruction (rows are
        // 16-byte aligned: the row stride ldbo is a multiple of 4)
        for (int e0 = 0; e0 < SW_ROWS * U; e0 += 32) {
            const int e = e0 + lane, r = e / U, u = e - r * U;
            const int kr = __shfl_sync(0xffffffffu, k, r < SW_ROWS ? r : 0);
            if (r < rows) {
                cp_async<16>(bo + r * MP + 2 * u, Bo + (size_t)kr * ldbo + 2 * u);
            }
        }
        // B, Bx (sorted per candidate) and x: coalesced, lanes over rows
        float *rw = sraw4 + (size_t)sg * RAW;
        const int i = i0 + lane;
        const bool ok = lane < rows;
        for (int cw = 0; cw < task.count; ++cw) {
            cp_async4(rw + cw * SW_ROWS + lane, bsb + (size_t)cw * n + (ok ? i : 0), ok);
            cp_async4(rw + (W + cw) * SW_ROWS + lane, bxb + (size_t)cw * n + (ok ? i : 0), ok);
        }
        cp_async4(rw + 2 * W * SW_ROWS + 1 + lane, xs + (ok ? i : 0), ok);
        if (lane == 0) {
            cp_async4(rw + 2 * W * SW_ROWS, xs + (i0 > 0 ? i0 - 1 : 0), i0 > 0);
        }
    };
    auto convert = [&](int sq) {  // stage sq (landed) -> f64 slot sq & 1, lanes over rows
        const float *rw = sraw4 + (size_t)(sq % S) * RAW;
        double *cv = scvt + (size_t)(sq & 1) * NV * SW_ROWS;
        for (int cw = 0; cw < task.count; ++cw) {
            cv[cw * SW_ROWS + lane] = (double)rw[cw * SW_ROWS + lane];
            cv[(W + cw) * SW_ROWS + lane] = (double)rw[(W + cw) * SW_ROWS + lane];
        }
        const float *xr = rw + 2 * W * SW_ROWS;  // xr[r] = x of row i0 + r - 1
        cv[2 * W * SW_ROWS + lane] =
            sq * SW_ROWS + lane > 0 ? (double)(xr[lane] - xr[lane + 1]) : 0.0;
    };

    const int mycand = task.cand0 + (cwarp ? wc : 0);
    const double ybx_c = part ? 0.0 : ybx[mycand];
    const double *mysc = scal + (size_t)mycand * ngrid * 3;
    double *snap = snapbase + (size_t)(cwarp ? wc : 0) * SW_SNAP * ldF;
    double f[CPL], g[CPL];
#pragma unroll
    for (int q = 0; q < CPL; ++q) {
        f[q] = 0.0;
        g[q] = 0.0;
    }
    double best = 0.0;
    int besti = -1;
    int nsnap = 0;  // block-uniform
    int next_grid = head + 1;

    auto flush = [&]() {
        if (cwarp && sub == 0) {
            double sse = -1.0;
            int row = 0x7fffffff;
            if (lane < nsnap) {
                row = srow[lane];
                const double *sc = mysc + (size_t)((row - (head + 1)) / min_span) * 3;
                const double k0 = sc[0], k1 = sc[1], w = sc[2];
                const double *fs = snap + (size_t)lane * ldF;
                double ff = 0.0, fy = 0.0;
                for (int c = 0; c < m; ++c) {
                    ff = fma(fs[c], fs[c], ff);
                    fy = fma(fs[c], sybo[c], fy);
                }
                ff = fma(fs[m], fs[m], ff);
                const double den = (k0 + k1) - ff;
                if (part) {
                    double *o = part + ((size_t)mycand * ngrid +
                                        (size_t)((row - (head + 1)) / min_span)) * 4;
                    o[0] = fy;
                    o[1] = fs[m];
                    o[2] = w;
                    o[3] = den;
                } else {
                    fy = fma(fs[m], ybx_c, fy);
                    const double uw = fy - w;
                    sse = den > tol ? (uw * uw) / (den + tol) : 0.0;
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
    };

    if (lwarp) {
        prefetch(0);
#pragma unroll
        for (int q = 0; q < S - 1; ++q) {
            if (q < nstages) {
                issue(q);
            }
            cp_async_commit();
            prefetch(q + 1);
        }
        cp_async_wait<S - 2>();  // stage 0 landed
        __syncwarp();
        if (nstages > 0) {
            convert(0);
        }
    }
    __syncthreads();
    for (int sq = 0; sq < nstages; ++sq) {
        const int sg = sq % S, h = sq & 1, i0 = sq * SW_ROWS;
        const int rows = min(SW_ROWS, tail - i0);
        int gcount = 0;
        unsigned gmask = 0u;  // the grid rows of this stage
        for (int gr = next_grid; gr < i0 + rows; gr += min_span) {
            gmask |= 1u << (gr - i0);
            ++gcount;
        }
        if (nsnap + gcount > SW_SNAP) {
            flush();
            __syncthreads();  // slots are rewritten below
        }
        if (cwarp) {
            const double *cv = scvt + (size_t)h * NV * SW_ROWS;
            const double *bw = cv + wc * SW_ROWS;
            const double *xw = cv + (W + wc) * SW_ROWS;
            const double *dv = cv + 2 * W * SW_ROWS;
            const double *rowb = sbo + (size_t)sg * SW_ROWS * MP;
            int slot = nsnap;
            auto step = [&](int r) {
                const double bk = bw[r], bxk = xw[r];
                const double *rowp = rowb + r * MP;
                const double di = dv[r];  // 0 for the first row
#pragma unroll
                for (int q = 0; q < CPL; ++q) {
                    const int c = lane + 32 * (sub + split * q);
                    const double bv = rowp[min(c, m - 1)];  // unconditional load, then select
                    const double xv = c < m ? bv : (c == m ? bxk : 0.0);
                    f[q] = fma(di, g[q], f[q]);
                    g[q] = fma(bk, xv, g[q]);
                }
                if (gmask & (1u << r)) {
                    double *fs = snap + (size_t)slot * ldF;
#pragma unroll
                    for (int q = 0; q < CPL; ++q) {
                        const int c = lane + 32 * (sub + split * q);
                        if (c <= m) {
                            fs[c] = f[q];
                        }
                    }
                    if (lane == 0 && warp == 0) {
                        srow[slot] = i0 + r;
                    }
                    ++slot;
                }
            };
            if (rows == SW_ROWS) {  // a whole stage, unrolled
#pragma unroll
                for (int r = 0; r < SW_ROWS; ++r) {
                    step(r);
                }
            } else {
                for (int r = 0; r < rows; ++r) {
                    step(r);
                }
            }
        } else if (lwarp) {
            if (sq + S - 1 < nstages) {
                issue(sq + S - 1);  // into the ring slot of stage sq - 1 (consumed)
            }
            cp_async_commit();
            prefetch(sq + S);
            cp_async_wait<S - 2>();  // stage sq + 1 landed
            __syncwarp();
            if (sq + 1 < nstages) {
                convert(sq + 1);
            }
        }
        nsnap += gcount;
        next_grid += gcount * min_span;
        __syncthreads();
    }
    if (nsnap > 0) {
        flush();
    }
    if (cwarp && sub == 0 && lane == 0 && !part) {
        hsse[mycand] = best;
        hrow[mycand] = besti >= 0 ? pk[besti] : -1;
    }
}

constexpr int SS_THREADS = 256;

__global__ void __launch_bounds__(SS_THREADS)
    k_sweep_score(const double *__restrict__ part, int ngrid, const int *__restrict__ cand_x,
                  const int *__restrict__ perm, const double *__restrict__ ybx, int n, int head,
                  int min_span, double tol, double *__restrict__ hsse, int *__restrict__ hrow)
{
    __shared__ double rs[SS_THREADS / 32];
    __shared__ int rg[SS_THREADS / 32];
    const int j = blockIdx.x;
    const double yb = ybx[j];
    const double *pj = part + (size_t)j * ngrid * 4;
    double best = -1.0;
    int bg = 0x7fffffff;
    for (int g = threadIdx.x; g < ngrid; g += SS_THREADS) {
        const double *q = pj + (size_t)g * 4;
        const double fy = fma(q[1], yb, q[0]);
        const double uw = fy - q[2];
        const double den = q[3];
        const double sse = den > tol ? (uw * uw) / (den + tol) : 0.0;
        if (sse > best) {  // g increases along a thread's loop: ties keep the first
            best = sse;
            bg = g;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double s2 = __shfl_xor_sync(0xffffffffu, best, o);
        const int g2 = __shfl_xor_sync(0xffffffffu, bg, o);
        if (s2 > best || (s2 == best && g2 < bg)) {
            best = s2;
            bg = g2;
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        rs[warp] = best;
        rg[warp] = bg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        best = rs[0];
        bg = rg[0];
        for (int w = 1; w < SS_THREADS / 32; ++w) {
            if (rs[w] > best || (rs[w] == best && rg[w] < bg)) {
                best = rs[w];
                bg = rg[w];
            }
        }
        // the reference keeps the first strictly positive maximum
        if (best > 0.0) {
            hsse[j] = best;
            hrow[j] = perm[(size_t)cand_x[j] * n + head + 1 + (size_t)bg * min_span];
        } else {
            hsse[j] = 0.0;
            hrow[j] = -1;
        }
    }
}

// ---------------------------------------------------------------------------
// The hinge sweep's scalar recurrences (marsalgo.cc:91-151 covariates_impl,
// used at :603-626): per row i >= 1 of the descending sort, with the previous
// row's values on the right-hand sides,
//   k0 += d^2 b2;  k1 += 2d bd;  w += d vb;  bd += d b2;  b2 += bk^2;  vb += yk bk,
// and vb = bk yk, b2 = bk^2 on the first row. They depend on the parent
// column, y and the sorted input only -- not on the basis or the candidate
// column -- so they run here, concurrently with the projection, and the sweep
// reads k0, k1, w at its grid rows.
//
// Block = one input column and up to 32 parents (lane = parent). GB300's FP64
// pipe takes one warp instruction per ~64 cycles per SM sub-partition, so no
// warp (one per sub-partition) issues more than two FMAs per row:
//   warp 0: vb, w      warp 1: b2, bd      warp 2: k0, k1
// Warp 1 leaves b2 and bd of every row in shared memory; warp 2 runs one
// stage (32 rows) behind and reads them there, long after they were written.
// Warp 3 stages the rows with coalesced cp.async from the sorted copies (the
// parents' B per candidate, y and x per input column) and converts them to
// f64 once, with the deltas (kept three stages deep for the lagging warp).
// Output per candidate and grid row g: scal[(cand * ngrid + g) * 3 + {0,1,2}] =
// k0, k1, w.
// ---------------------------------------------------------------------------
constexpr int SC_ROWS = 32, SC_STAGES = 4, SC_THREADS = 128, SC_MAXP = 32;

// Dynamic shared memory of k_hinge_scalars (byte offsets).
struct ScSmem {
    static constexpr size_t rb = 0;  // [S][MAXP][ROWS] f32, B of each parent, lanes over rows
    static constexpr size_t ry = rb + 4 * SC_STAGES * SC_MAXP * SC_ROWS;  // [S][ROWS] f32
    static constexpr size_t rx = ry + 4 * SC_STAGES * SC_ROWS;  // [S][ROWS + 1] f32
    static constexpr size_t db = align16(rx + 4 * SC_STAGES * (SC_ROWS + 1));  // [2][ROWS][MAXP+1]
    static constexpr size_t dy = db + 8 * 2 * SC_ROWS * (SC_MAXP + 1);  // [2][ROWS] f64
    static constexpr size_t sd = dy + 8 * 2 * SC_ROWS;    // [3][ROWS] f64: d, then d^2, 2d
    static constexpr size_t sdd = sd + 8 * 3 * SC_ROWS;
    static constexpr size_t sd2 = sdd + 8 * 3 * SC_ROWS;
    static constexpr size_t lb2 = sd2 + 8 * 3 * SC_ROWS;  // [2][ROWS][MAXP] f64, b2 after row r
    static constexpr size_t lbd = lb2 + 8 * 2 * SC_ROWS * SC_MAXP;  // bd after row r
    static constexpr size_t total = lbd + 8 * 2 * SC_ROWS * SC_MAXP;
};

__global__ void __launch_bounds__(SC_THREADS)
    k_hinge_scalars(const SweepTask *__restrict__ tasks, const float *__restrict__ xsort,
                    const float *__restrict__ ysort, const float *__restrict__ bs, int n,
                    int head, int tail, int min_span, int ngrid, double *__restrict__ scal)
{
    constexpr int S = SC_STAGES;
    extern __shared__ __align__(16) unsigned char scm[];
    auto rb = reinterpret_cast<float(*)[SC_MAXP][SC_ROWS]>(scm + ScSmem::rb);
    auto ry = reinterpret_cast<float(*)[SC_ROWS]>(scm + ScSmem::ry);
    auto rx = reinterpret_cast<float(*)[SC_ROWS + 1]>(scm + ScSmem::rx);
    auto db = reinterpret_cast<double(*)[SC_ROWS][SC_MAXP + 1]>(scm + ScSmem::db);
    auto dy = reinterpret_cast<double(*)[SC_ROWS]>(scm + ScSmem::dy);
    auto sd = reinterpret_cast<double(*)[SC_ROWS]>(scm + ScSmem::sd);
    auto sdd = reinterpret_cast<double(*)[SC_ROWS]>(scm + ScSmem::sdd);
    auto sd2 = reinterpret_cast<double(*)[SC_ROWS]>(scm + ScSmem::sd2);
    auto lb2 = reinterpret_cast<double(*)[SC_ROWS][SC_MAXP]>(scm + ScSmem::lb2);
    auto lbd = reinterpret_cast<double(*)[SC_ROWS][SC_MAXP]>(scm + ScSmem::lbd);

    const SweepTask task = tasks[blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float *xs = xsort + (size_t)task.xcol * n;
    const float *ys = ysort + (size_t)task.xcol * n;
    const float *bsb = bs + (size_t)task.cand0 * n;
    const int nstages = (tail + SC_ROWS - 1) / SC_ROWS;
    const bool lwarp = warp == 3;

    auto issue = [&](int sq) {
        const int sg = sq % S, i0 = sq * SC_ROWS, i = i0 + lane;
        const bool ok = i < tail;
        for (int q = 0; q < task.count; ++q) {
            cp_async4(&rb[sg][q][lane], bsb + (size_t)q * n + (ok ? i : 0), ok);
        }
        cp_async4(&ry[sg][lane], ys + (ok ? i : 0), ok);
        cp_async4(&rx[sg][lane + 1], xs + (ok ? i : 0), ok);
        if (lane == 0) {
            cp_async4(&rx[sg][0], xs + (i0 > 0 ? i0 - 1 : 0), i0 > 0);
        }
    };
    // stage sq (landed) -> f64: B and y in slot sq & 1, the deltas in slot sq % 3
    auto convert = [&](int sq) {
        const int sg = sq % S, h = sq & 1, h3 = sq % 3, i = sq * SC_ROWS + lane;
        for (int q = 0; q < task.count; ++q) {
            db[h][lane][q] = (double)rb[sg][q][lane];
        }
        dy[h][lane] = (double)ry[sg][lane];
        const double dl = i > 0 ? (double)(rx[sg][lane] - rx[sg][lane + 1]) : 0.0;
        sd[h3][lane] = dl;
        sdd[h3][lane] = dl * dl;
        sd2[h3][lane] = dl * 2;
    };

    if (lwarp) {
#pragma unroll
        for (int q = 0; q < S - 1; ++q) {
            if (q < nstages) {
                issue(q);
            }
            cp_async_commit();
        }
        cp_async_wait<S - 2>();
        __syncwarp();
        if (nstages > 0) {
            convert(0);
        }
    }
    __syncthreads();
    const bool active = !lwarp && lane < task.count;
    double *out = scal + (size_t)(task.cand0 + (lane < task.count ? lane : 0)) * ngrid * 3;
    // role 0: v0 = vb, v1 = w; role 1: v0 = b2, v1 = bd; role 2: v0 = k0, v1 = k1,
    // one stage behind roles 0 and 1, from the b2 and bd they leave per row
    double v0 = 0.0, v1 = 0.0;
    double pb2 = 0.0, pbd = 0.0;  // role 2: b2 and bd after the row before its stage
    int gi = 0;
    auto grid_mask = [&](int ng, int i0, int rows) {
        unsigned mask = 0u;
        for (int g = ng; g < i0 + rows; g += min_span) {
            mask |= 1u << (g - i0);
        }
        return mask;
    };
    auto stage = [&](auto role, int sq, int rows, unsigned gmask) {
        constexpr int R = decltype(role)::value;
        const int i0 = sq * SC_ROWS, h = sq & 1, h3 = sq % 3;
        const double *dv = sd[h3], *ddv = sdd[h3], *d2v = sd2[h3];
        auto step = [&](int r) {
            const int i = i0 + r;
            if (R == 0) {  // vb, w
                const double bk = db[h][r][lane], yk = dy[h][r];
                if (i == 0) {
                    v0 = bk * yk;
                } else {
                    v1 = fma(dv[r], v0, v1);
                    v0 = fma(yk, bk, v0);
                }
            } else if (R == 1) {  // b2, bd
                const double bk = db[h][r][lane];
                if (i == 0) {
                    v0 = bk * bk;
                } else {
                    v1 = fma(dv[r], v0, v1);
                    v0 = fma(bk, bk, v0);
                }
                lb2[h][r][lane] = v0;
                lbd[h][r][lane] = v1;
            } else {  // k0, k1 from the b2 and bd after the previous row
                const double b2p = r == 0 ? pb2 : lb2[h][r - 1][lane];
                const double bdp = r == 0 ? pbd : lbd[h][r - 1][lane];
                if (i > 0) {
                    v0 = fma(ddv[r], b2p, v0);
                    v1 = fma(d2v[r], bdp, v1);
                }
            }
            if (R != 1 && (gmask & (1u << r))) {
                double *o = out + (size_t)gi * 3;
                if (R == 0) {
                    o[2] = v1;
                } else {
                    o[0] = v0;
                    o[1] = v1;
                }
                ++gi;
            }
        };
        if (rows == SC_ROWS) {  // a whole stage, unrolled
#pragma unroll
            for (int r = 0; r < SC_ROWS; ++r) {
                step(r);
            }
        } else {
            for (int r = 0; r < rows; ++r) {
                step(r);
            }
        }
        if (R == 2) {
            pb2 = lb2[h][rows - 1][lane];
            pbd = lbd[h][rows - 1][lane];
        }
    };
    int ng = head + 1, ng2 = head + 1;  // next grid row of stage sq, and of stage sq - 1
    for (int sq = 0; sq <= nstages; ++sq) {
        const int rows = sq < nstages ? min(SC_ROWS, tail - sq * SC_ROWS) : 0;
        const unsigned gmask = sq < nstages ? grid_mask(ng, sq * SC_ROWS, rows) : 0u;
        const int rows2 = sq > 0 ? min(SC_ROWS, tail - (sq - 1) * SC_ROWS) : 0;
        const unsigned gmask2 = sq > 0 ? grid_mask(ng2, (sq - 1) * SC_ROWS, rows2) : 0u;
        const int gc = __popc(gmask), gc2 = __popc(gmask2);
        if (active) {
            if (warp == 0 && sq < nstages) {
                stage(std::integral_constant<int, 0>(), sq, rows, gmask);
            } else if (warp == 1 && sq < nstages) {
                stage(std::integral_constant<int, 1>(), sq, rows, gmask);
            } else if (warp == 2 && sq > 0) {
                stage(std::integral_constant<int, 2>(), sq - 1, rows2, gmask2);
            }
        } else if (lwarp && sq < nstages) {
            if (sq + S - 1 < nstages) {
                issue(sq + S - 1);
            }
            cp_async_commit();
            cp_async_wait<S - 2>();
            __syncwarp();
            if (sq + 1 < nstages) {
                convert(sq + 1);
            }
        }
        ng += gc * min_span;
        ng2 += gc2 * min_span;
        __syncthreads();
    }
}

// The same scalars, exact and parallel over the rows (xhinge.cuh): one block
// per candidate (blockIdx.x the task, blockIdx.y its candidate), one chunk of L
// consecutive rows per thread. Per level: float-float guesses of every chunk's
// entry values from a block scan, XC_RUNS speculative runs per chain (thread 0
// runs chunk 0 from the true start), then one thread per chain walks the chunks
// (different warps, so the walks overlap). Last, every thread re-runs its chunk
// from the exact entry values and writes k0, k1, w at its grid rows. The values
// equal those of k_hinge_scalars bit for bit.
constexpr int XH_MAXK = 512;

size_t xh_smem_bytes(int K)
{
    return sizeof(XcChunk) * 3 * (size_t)K + sizeof(double) * (XS_N * (size_t)K + XH_MAXK / 32);
}

// Exclusive prefix over the block's threads of v (a guess: rounding is harmless).
__device__ double xh_block_prefix(double v, double *wsum)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) {
            inc += u;
        }
    }
    __syncthreads();  // wsum of the previous call has been read
    if (lane == 31) {
        wsum[warp] = inc;
    }
    __syncthreads();
    if (warp == 0) {
        double w = lane < nw ? wsum[lane] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) {
                w += u;
            }
        }
        if (lane < nw) {
            wsum[lane] = w;
        }
    }
    __syncthreads();
    return (inc - v) + (warp > 0 ? wsum[warp - 1] : 0.0);
}

// Chain j's walk over chunks 1 .. K-2: st[j][c + 1] from st[j][c] and the
// chunk's record; M is the set of chains a re-run of the chunk needs.
template <int M>
__device__ void xh_walk(const XhRows &R, int j, const XcChunk *rec, double *st, int K, int L,
                        int tail)
{
    for (int c = 1; c + 1 < K; ++c) {
        const int c0 = min(tail, c * L), c1 = min(tail, c0 + L);
        bool redone = false;
        st[j * K + c + 1] = xc_resolve_with(rec[c], st[j * K + c], [&](double v) {
            XhState s;
#pragma unroll
            for (int q = 0; q < XS_N; ++q) {
                s.v[q] = st[q * K + c];
            }
            s.v[j] = v;
            xh_run<M>(R, c0, c1, s);
            return s.v[j];
        }, &redone);
    }
}

__global__ void __launch_bounds__(XH_MAXK)
    k_hinge_xscalars(const SweepTask *__restrict__ tasks, const float *__restrict__ xsort,
                     const float *__restrict__ ysort, const float *__restrict__ bs, int n,
                     int head, int tail, int min_span, int ngrid, double *__restrict__ scal)
{
    const SweepTask task = tasks[blockIdx.x];
    const int q = blockIdx.y;
    if (q >= task.count) {
        return;  // the whole block
    }
    extern __shared__ __align__(16) unsigned char xsm[];
    const int K = blockDim.x, t = threadIdx.x;
    XcChunk *ch = reinterpret_cast<XcChunk *>(xsm);                                  // [3][K]
    double *st = reinterpret_cast<double *>(xsm + sizeof(XcChunk) * 3 * (size_t)K);  // [XS_N][K]
    double *wsum = st + XS_N * K;
    const int cand = task.cand0 + q;
    const XhRows R{bs + (size_t)cand * n, ysort + (size_t)task.xcol * n,
                   xsort + (size_t)task.xcol * n};
    const int L = (tail + K - 1) / K;
    const int i0 = (int)min((long long)tail, (long long)t * L), i1 = min(tail, i0 + L);
    const int w1 = 32 < K ? 32 : 0, w2 = 64 < K ? 64 : 0;  // walkers of chains 1 and 2
#pragma unroll
    for (int j = 0; j < XS_N; ++j) {
        st[j * K + t] = 0.0;
    }
    double g[3], gp[3];

    // level 1: b2, vb
    xh_guess1(R, i0, i1, g);
    gp[0] = xh_block_prefix(g[0], wsum);
    gp[1] = xh_block_prefix(g[1], wsum);
    if (t == 0) {
        XhState s{};
        xh_run<XH_B2 | XH_VB>(R, i0, i1, s);
        if (K > 1) {
            st[XS_B2 * K + 1] = s.v[XS_B2];
            st[XS_VB * K + 1] = s.v[XS_VB];
        }
    } else {
        xh_spec1(R, i0, i1, gp, ch + t, K);
    }
    __syncthreads();
    if (t == 0) {
        xh_walk<XH_B2>(R, XS_B2, ch, st, K, L, tail);
    }
    if (t == w1) {
        xh_walk<XH_VB>(R, XS_VB, ch + K, st, K, L, tail);
    }
    __syncthreads();

    // level 2: bd, w, k0
    xh_guess2(R, i0, i1, st[XS_B2 * K + t], st[XS_VB * K + t], g);
    gp[0] = xh_block_prefix(g[0], wsum);
    gp[1] = xh_block_prefix(g[1], wsum);
    gp[2] = xh_block_prefix(g[2], wsum);
    if (t == 0) {
        XhState s{};
        xh_run<XH_B2 | XH_VB | XH_BD | XH_W | XH_K0>(R, i0, i1, s);
        if (K > 1) {
            st[XS_BD * K + 1] = s.v[XS_BD];
            st[XS_W * K + 1] = s.v[XS_W];
            st[XS_K0 * K + 1] = s.v[XS_K0];
        }
    } else {
        xh_spec2(R, i0, i1, st[XS_B2 * K + t], st[XS_VB * K + t], gp, ch + t, K);
    }
    __syncthreads();
    if (t == 0) {
        xh_walk<XH_B2 | XH_BD>(R, XS_BD, ch, st, K, L, tail);
    }
    if (t == w1) {
        xh_walk<XH_VB | XH_W>(R, XS_W, ch + K, st, K, L, tail);
    }
    if (t == w2) {
        xh_walk<XH_B2 | XH_K0>(R, XS_K0, ch + 2 * K, st, K, L, tail);
    }
    __syncthreads();

    // level 3: k1
    xh_guess3(R, i0, i1, st[XS_B2 * K + t], st[XS_BD * K + t], g);
    gp[0] = xh_block_prefix(g[0], wsum);
    if (t == 0) {
        XhState s{};
        xh_run<XH_B2 | XH_BD | XH_K1>(R, i0, i1, s);
        if (K > 1) {
            st[XS_K1 * K + 1] = s.v[XS_K1];
        }
    } else {
        xh_spec3(R, i0, i1, st[XS_B2 * K + t], st[XS_BD * K + t], gp, ch + t);
    }
    __syncthreads();
    if (t == 0) {
        xh_walk<XH_B2 | XH_BD | XH_K1>(R, XS_K1, ch, st, K, L, tail);
    }
    __syncthreads();

    // the grid rows of this thread's chunk
    XhState s;
#pragma unroll
    for (int j = 0; j < XS_N; ++j) {
        s.v[j] = st[j * K + t];
    }
    double *out = scal + (size_t)cand * ngrid * 3;
    xh_output(R, i0, i1, s, head, min_span, [&](int gq, double k0, double k1, double w) {
        out[(size_t)gq * 3] = k0;
        out[(size_t)gq * 3 + 1] = k1;
        out[(size_t)gq * 3 + 2] = w;
    });
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
                                const float *__restrict__ y, int n, int col,
                                const int *__restrict__ perm, float *__restrict__ xsort,
                                float *__restrict__ ysort)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int k = perm[i];
        xsort[i] = X[k + (size_t)col * ldX] * s[col];
        ysort[i] = y[k];
    }
}

// Per candidate j, its parent column B[:, cand_b[j]] in the descending order
// of its input column: bs[j * n + i] = B[perm_x[i], cand_b[j]], i < rows.
__global__ void k_gather_parent(const int *__restrict__ perm, const float *__restrict__ B,
                                size_t ldB, const int *__restrict__ cand_x,
                                const int *__restrict__ cand_b, int n, int rows, int P,
                                float *__restrict__ bs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (int j = blockIdx.y; j < P; j += gridDim.y) {
        if (i < rows) {
            const int k = perm[(size_t)cand_x[j] * n + i];
            bs[(size_t)j * n + i] = B[(size_t)k + (size_t)cand_b[j] * ldB];
        }
    }
}

// Per candidate j, its normalised column in the descending order of its
// input column: bxs[j * n + i] = Bx[perm_x[i], j] * scale_j (the f32 product
// of kernels.cc:401-416).
__global__ void k_gather_scaled_candidate(const int *__restrict__ perm,
                                          const float *__restrict__ Bx, size_t ldBx,
                                          const int *__restrict__ cand_x,
                                          const double *__restrict__ s, double tol, int n,
                                          int rows, int P, float *__restrict__ bxs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (int j = blockIdx.y; j < P; j += gridDim.y) {
        const float sc = norm_scale(s[j], tol);
        if (i < rows) {
            const int k = perm[(size_t)cand_x[j] * n + i];
            bxs[(size_t)j * n + i] = Bx[(size_t)k + (size_t)j * ldBx] * sc;
        }
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

}  // namespace


template <class Src, class BoT>
void tgemm_fp64(cudaStream_t st, const Src &src, const BoT *Bo, size_t ldbo, int n, int m, int P,
                double *T, long long *launches)
{
    if (P <= 0 || m <= 0) {
        return;
    }
    int kt = 4;
    while (kt < m && kt < 32) {
        kt *= 2;
    }
    const unsigned gx = (unsigned)ceil_div(m, kt), gy = (unsigned)ceil_div(P, TG_THREADS / kt);
    verify(gy <= 65535, "too many candidate columns for one launch", 2);
#define TG_CASE(K)                                                                           \
    case K: {                                                                                \
        const size_t smem = TgemmSmem<BoT, K, Src::kRaw>::total;                             \
        if (smem > 48 * 1024) {                                                              \
            allow_smem(k_tgemm<Src, BoT, K>, smem);                                            \
        }                                                                                    \
        k_tgemm<Src, BoT, K><<<dim3(gx, gy), TG_THREADS, smem, st>>>(src, Bo, ldbo, n, m, P, T); \
        break;                                                                               \
    }
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

#define TG_INST(SRC, BOT)                                                                     \
    template void tgemm_fp64<SRC, BOT>(cudaStream_t, const SRC &, const BOT *, size_t, int, int, \
                                       int, double *, long long *);
TG_INST(FillSrc, float)
TG_INST(FillSrc, double)
TG_INST(StoredSrc, float)
TG_INST(StoredSrc, double)
#undef TG_INST

// Chunks per chain for k_xchain, or 0 where the chains as written (k_colchain,
// k_tgemm) are the faster form. Costs in SM cycles over the GPU: a chain as
// written takes plain_step cycles a row (~70 for a column chain, ~86 for a T
// chain with its operand load); FP64 throughput is ~2 FMAs per cycle per SM;
// k_xchain issues XC_RUNS + 1 FMAs per element (the runs from the guess and
// from zero) and its walk takes ~450 cycles a chunk. MARS_GPU_XCHAIN = 0 or 1
// forces either form.
int xchain_chunks(int n, int P, double plain_step)
{
    const char *fv = std::getenv("MARS_GPU_XCHAIN");
    const int force = fv && *fv ? std::atoi(fv) : -1;
    if (n <= 0 || force == 0) {
        return 0;
    }
    const int K = (int)std::min<size_t>(XC_MAXK, std::max<size_t>(32, round_up(ceil_div(n, 2048), 32)));
    if (force == 1) {
        return K;
    }
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    const double fp64 = 2.0 * std::max(1, sms);
    const double plain = std::max(plain_step * n, (double)P * n / fp64);
    const double chunked = (XC_RUNS + 1.0) * P * n / fp64 + 450.0 * K;
    return chunked < 0.7 * plain ? K : 0;
}

template <class Op>
void colchain(cudaStream_t st, const Op &op, int n, int P, double *out, long long *launches)
{
    if (P <= 0) {
        return;
    }
    const int K = xchain_chunks(n, P, 70.0);
    if (K > 0) {
        k_xchain<ColChains<Op>><<<(unsigned)P, (unsigned)K, 0, st>>>(ColChains<Op>{op}, n,
                                                                    (int)ceil_div(n, K), out);
    } else {
        k_colchain<Op><<<(unsigned)ceil_div(P, CC_COLS), CC_THREADS, 0, st>>>(op, n, P, out);
    }
    LAUNCH_CHECK();
    *launches += 1;
}

template <class Src, class BoT>
void project_fp64(cudaStream_t st, const Src &src, const BoT *Bo, size_t ldbo, const float *BoC,
                  XaBufs *xa, int n, int m, int P, const int *out_col, float *Bx, size_t ldBx,
                  double *s_out, const ProjectScratch &ws, long long *launches)
{
    if (P <= 0) {
        return;
    }
    // A chain as written costs ~86 cycles a row whatever the number of chains.
    // The exact parallel form reads both columns of every chain (no reuse
    // across chains) with strided per-thread rows: measured at 10^6 rows, 1,012
    // chains take 39 ms against 57 ms as written and 1,472 take 56 ms, so it
    // is taken up to 1,200 chains.
    bool done = false;
    if constexpr (std::is_same<Src, StoredSrc>::value) {
        if (BoC && xa && m > 0 && n >= 65536 && (long long)P * m <= 1200) {
            done = tgemm_exact(st, n, m, P, BoC, src.Bx, src.ldBx, src.col, ws.T, *xa, launches);
        }
    }
    if (!done) {
        tgemm_fp64(st, src, Bo, ldbo, n, m, P, ws.T, launches);
    }
    const int rb = (int)ceil_div(n, PJ_THREADS);
    const size_t smem = sizeof(double) * PJ_COLS * std::max(m, 1);
    if (smem > 48 * 1024) {
        allow_smem(k_project<Src, BoT>, smem);
    }
    verify(ceil_div(P, PJ_COLS) <= 65535, "too many candidate columns for one launch", 2);
    k_project<Src, BoT><<<dim3(rb, (unsigned)ceil_div(P, PJ_COLS)), PJ_THREADS, smem, st>>>(
        src, Bo, ldbo, n, m, P, ws.T, out_col, Bx, ldBx);
    LAUNCH_CHECK();
    *launches += 1;
    colchain(st, SqChain{Bx, ldBx, out_col}, n, P, s_out, launches);
}

#define PJ_INST(SRC, BOT)                                                                      \
    template void project_fp64<SRC, BOT>(cudaStream_t, const SRC &, const BOT *, size_t,       \
                                         const float *, XaBufs *, int, int, int, const int *,   \
                                         float *, size_t, double *, const ProjectScratch &,     \
                                         long long *);
PJ_INST(FillSrc, float)
PJ_INST(FillSrc, double)
PJ_INST(StoredSrc, float)
PJ_INST(StoredSrc, double)
#undef PJ_INST

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
// candidates (two blocks per SM) or the snapshots would not fit; the row ring
// is 4 stages deep when it fits in 200 KB with the snapshots, else 2.
static size_t sweep_smem(int m, int w, int stages) { return SweepSmem(m, w, stages).total; }

int sweep_split(int m, int candidates)
{
    // More than 32 components put 2 FMAs per component slot and row on a
    // warp; with few candidates (the sweep is then a latency-bound walk, not
    // FP64-pipe bound) two warps share each candidate instead.
    return m + 1 > 32 && candidates <= 2 * 152 ? 2 : 1;
}

int sweep_warps(int m, int candidates)
{
    // Each candidate warp issues two dependent FP64 FMAs per row and an SM
    // sub-partition's FP64 pipe takes one warp instruction per ~64 cycles, so
    // a candidate warp wants a sub-partition of its own: 4 candidate warps per
    // block (warps map to sub-partitions by index mod 4; the light loader
    // shares one), one block per SM up to 4 x 152 candidates, then 5.
    // Returns candidates per block: warps / sweep_split.
    const int split = sweep_split(m, candidates);
    int w = candidates <= 4 * 152 ? 4 : SW_MAXW;
    while (w > split && sweep_smem(m, w, 2) > 200 * 1024) {
        --w;
    }
    return std::max(1, w / split);
}

int sweep_grid_rows(int head, int tail, int min_span)
{
    return tail - 1 >= head + 1 ? (tail - 1 - (head + 1)) / min_span + 1 : 0;
}

void gather_parents(cudaStream_t st, const int *perm, const float *B, size_t ldB,
                    const int *cand_x, const int *cand_b, int n, int rows, int P, float *bs,
                    long long *launches)
{
    if (P <= 0 || rows <= 0) {
        return;
    }
    const dim3 grid((unsigned)ceil_div(rows, 256), (unsigned)std::min(P, 65535));
    k_gather_parent<<<grid, 256, 0, st>>>(perm, B, ldB, cand_x, cand_b, n, rows, P, bs);
    LAUNCH_CHECK();
    *launches += 1;
}

void gather_candidates(cudaStream_t st, const int *perm, const float *Bx, size_t ldBx,
                       const int *cand_x, const double *s, double tol, int n, int rows, int P,
                       float *bxs, long long *launches)
{
    if (P <= 0 || rows <= 0) {
        return;
    }
    const dim3 grid((unsigned)ceil_div(rows, 256), (unsigned)std::min(P, 65535));
    k_gather_scaled_candidate<<<grid, 256, 0, st>>>(perm, Bx, ldBx, cand_x, s, tol, n, rows, P,
                                                    bxs);
    LAUNCH_CHECK();
    *launches += 1;
}

// Threads (chunks) per candidate for k_hinge_xscalars, or 0 where k_hinge_scalars
// is the better form. k_hinge_scalars advances a row per ~370 cycles and issues
// 6 FP64 FMAs per row and candidate; k_hinge_xscalars issues ~40 (the XC_RUNS
// runs and the run from zero of each chain, and the lower chains re-run beside
// them) on one SM per candidate, and walks its chunks three times at ~450 cycles
// a chunk. Both run beside the projection, whose FP64 chains they would slow
// down once the candidates outnumber the SMs: the chunked form is taken only
// for at most one candidate per SM, and where it is the faster of the two.
// MARS_GPU_XCHAIN = 0 or 1 forces either kernel.
int xh_chunks(int tail, int ncand)
{
    const char *fv = std::getenv("MARS_GPU_XCHAIN");
    const int force = fv && *fv ? std::atoi(fv) : -1;
    if (tail <= 0 || ncand <= 0 || force == 0) {
        return 0;
    }
    const int K = (int)std::min<size_t>(XH_MAXK, std::max<size_t>(32, round_up(ceil_div(tail, 1024), 32)));
    if (force == 1) {
        return K;
    }
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    if (ncand > sms) {
        return 0;
    }
    const double plain = 370.0 * tail;
    const double chunked = 40.0 * tail / 2.0 + 3 * 450.0 * K;
    return chunked < 0.7 * plain ? K : 0;
}

void hinge_scalars(cudaStream_t st, const SweepTask *tasks, int ntasks, int ncand,
                   const float *xsort, const float *ysort, const float *bs, int n, int head,
                   int tail, int min_span, double *scal, long long *launches)
{
    if (ntasks <= 0) {
        return;
    }
    const int K = xh_chunks(tail, ncand);
    if (K > 0) {
        const size_t smem = xh_smem_bytes(K);
        allow_smem(k_hinge_xscalars, smem);
        k_hinge_xscalars<<<dim3((unsigned)ntasks, 32), (unsigned)K, smem, st>>>(
            tasks, xsort, ysort, bs, n, head, tail, min_span,
            sweep_grid_rows(head, tail, min_span), scal);
        LAUNCH_CHECK();
        *launches += 1;
        return;
    }
    allow_smem(k_hinge_scalars, ScSmem::total);
    k_hinge_scalars<<<ntasks, SC_THREADS, ScSmem::total, st>>>(
        tasks, xsort, ysort, bs, n, head, tail, min_span, sweep_grid_rows(head, tail, min_span),
        scal);
    LAUNCH_CHECK();
    *launches += 1;
}

void sweep_fp64(cudaStream_t st, const SweepTask *tasks, int ntasks, const int *perm,
                const float *xsort, const float *bs, const float *bxs, const double *Bo,
                size_t ldbo, const double *ybo, const double *ybx, const double *scal, int n,
                int m, int head, int tail, int min_span, double tol, double *hsse, int *hrow,
                int warps_per_block, long long *launches, double *part, int split)
{
    if (ntasks <= 0) {
        return;
    }
    verify(split >= 1 && split <= 4, "sweep split out of range", 2);
    const int warps = warps_per_block * split;
    verify(warps >= 1 && warps <= SW_MAXW, "sweep block size out of range", 2);
    const int stages = sweep_smem(m, warps, 4) <= 200 * 1024 ? 4 : 2;
    const size_t smem = sweep_smem(m, warps, stages);
    if (smem > 227 * 1024) {
        int mmax = 1;
        while (sweep_smem(mmax + 1, 1, 2) <= 227 * 1024) {
            ++mmax;
        }
        throw Error(1, "the GPU hinge sweep supports at most " + std::to_string(mmax) +
                           " basis functions");
    }
    const int ngrid = sweep_grid_rows(head, tail, min_span);
    const int comps = (m + split) / split;  // components per warp: ceil((m + 1) / split)
#define LAUNCH_SWEEP(CPL, S)                                                                   \
    do {                                                                                       \
        allow_smem(k_sweep<CPL, S>, smem);                                                     \
        k_sweep<CPL, S><<<ntasks, 32 * (warps + 1), smem, st>>>(                               \
            tasks, perm, xsort, bs, bxs, Bo, ldbo, ybo, ybx, scal, ngrid, n, m, head, tail,    \
            min_span, tol, hsse, hrow, part, split);                                           \
    } while (0)
#define LAUNCH_CPL(CPL)            \
    do {                           \
        if (stages == 4) {         \
            LAUNCH_SWEEP(CPL, 4);  \
        } else {                   \
            LAUNCH_SWEEP(CPL, 2);  \
        }                          \
    } while (0)
    if (comps <= 32) {
        LAUNCH_CPL(1);
    } else if (comps <= 64) {
        LAUNCH_CPL(2);
    } else if (comps <= 128) {
        LAUNCH_CPL(4);
    } else if (comps <= 256) {
        LAUNCH_CPL(8);
    } else {
        LAUNCH_CPL(10);
    }
#undef LAUNCH_CPL
#undef LAUNCH_SWEEP
    LAUNCH_CHECK();
    *launches += 1;
}

void sweep_score(cudaStream_t st, const double *part, int P, const int *cand_x,
                 const int *perm, const double *ybx, int n, int head, int tail, int min_span,
                 double tol, double *hsse, int *hrow, long long *launches)
{
    if (P <= 0) {
        return;
    }
    const int ngrid = sweep_grid_rows(head, tail, min_span);
    k_sweep_score<<<P, SS_THREADS, 0, st>>>(part, ngrid, cand_x, perm, ybx, n, head, min_span,
                                            tol, hsse, hrow);
    LAUNCH_CHECK();
    *launches += 1;
}

void sort_columns(cudaStream_t st, const float *X, size_t ldX, const float *s, const float *y,
                  int n, const int *cols, int ncols, int *perm, float *xsort, float *ysort,
                  DevBuf &keys, DevBuf &vals, DevBuf &tmp, long long *launches)
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
        k_gather_scaled<<<nb, 256, 0, st>>>(X, ldX, s, y, n, c, pc, xsort + (size_t)c * n,
                                            ysort + (size_t)c * n);
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

// sum_i X[i,j]^2 per column as the reference's sequential fused chain
// (marsalgo.cc:359-369).
struct XSqChain {  // sum of squares of the X column j
    static constexpr bool kUsesY = false;
    const float *X;
    size_t ld;
    __device__ __forceinline__ const float *column(int j) const { return X + (size_t)j * ld; }
    __device__ __forceinline__ const float *ycolumn() const { return nullptr; }
    __device__ __forceinline__ float param(int) const { return 0.f; }
    __device__ __forceinline__ float value(float v, float) const { return v; }
    __device__ __forceinline__ double step(double acc, double v, double) const
    {
        return fma(v, v, acc);
    }
};

void column_sumsq(cudaStream_t st, const float *X, size_t ldX, int n, int p, double *out,
                  long long *launches)
{
    colchain(st, XSqChain{X, ldX}, n, p, out, launches);
}

}  // namespace mgpu
