// Tensor-core projection of the mixed-precision fast pass (tc.cuh).
//
// Two kernels, both issuing tcgen05.mma (kind::tf32, one elected thread per
// CTA, accumulators in tensor memory) with the FP32 operands split into two
// TF32 terms (3 products per K step, FP32 accumulation):
//
//   k_tc_tgemm    T^T (P x m) = src^T Bo: tile = 128 candidates x N = m
//                 padded to 16, K = the rows of one split of the n rows, 32 at
//                 a time. Bo (hi, lo) arrives by TMA from the column-major
//                 split copies; the candidate operand (hi, lo) is formed by
//                 eight producer warps from its source columns and written in
//                 the same 128-byte-swizzled K-major layout. Each 128-row
//                 chunk is summed in tensor memory and folded into FP32
//                 registers by drain warps; partials per split are summed in
//                 FP64 in a fixed order (k_tc_treduce).
//   k_tc_project  Bx (n x P) = src - Bo T: persistent, tile = 128 rows x 64
//                 candidates, K = m padded to 32; Bo rows (hi, lo) and T
//                 (hi, lo) both by TMA, two pairs of accumulators in tensor
//                 memory (hi*hi and the small hi*lo + lo*hi apart, so the
//                 truncating FP32 adds of the tensor cores see few large
//                 terms) so the epilogue of one tile overlaps the MMAs of the
//                 next; the epilogue subtracts from the source column and
//                 stores Bx column-major (coalesced across a warp's rows).
//
// Every wait on an mbarrier is bounded (about four seconds of global time):
// on expiry the waiting thread records MARS_GPU_ETIMEOUT in the error word,
// raises the block's abort flag, and every thread winds down to the common
// exit, where in-flight TMA copies and MMAs are waited for (again bounded)
// and the tensor memory is freed.
#include "tc.cuh"

#include "../../include/mars_gpu.h"
#include "fast.cuh"

#include <cuda.h>

#include <algorithm>
#include <mutex>

namespace mgpu {

namespace {

// ---------------------------------------------------------------------------
// PTX helpers (sm_100 family: mbarrier, TMA, tcgen05)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

constexpr unsigned long long TC_WAIT_NS = 4000000000ull;  // 4 s

// Waits for the phase of `bar` with parity `parity`. Returns false when the
// block is aborting (flag raised elsewhere) or when this wait ran out, in
// which case it raises the flag and records the error. With `drain` set the
// abort flag is ignored (used at exit to let in-flight work land).
__device__ __noinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                       int *err, bool drain = false)
{
    const unsigned long long t0 = global_ns();
    for (uint32_t it = 0;; ++it) {
        if (mbar_try(bar, parity)) {
            return true;
        }
        if (!drain && *abort_flag) {
            return false;
        }
        if ((it & 63) == 63) {
            if (global_ns() - t0 > TC_WAIT_NS) {
                *abort_flag = 1;
                atomicExch(err, MARS_GPU_ETIMEOUT);
                return false;
            }
            __nanosleep(128);
        }
    }
}

// mbar_wait by lane 0 of the warp, its result given to every lane.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t *bar, uint32_t parity,
                                               volatile int *abort_flag, int *err)
{
    bool ok = true;
    if ((threadIdx.x & 31) == 0) {
        ok = mbar_wait(bar, parity, abort_flag, err);
    }
    return __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap *map)
{
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// Whole warp: allocate `ncols` tensor-memory columns, address into *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr),
                 "r"(ncols)
                 : "memory");
}

// D[tmem] (+)= A[smem] * B[smem], kind::tf32, cta_group::1.
__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on `bar` once every MMA this thread issued so far has completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
            smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor: K-major operand in the canonical
// 128-byte-swizzled layout (rows of 128 bytes, 8-row atoms 1024 bytes apart).
// `addr` is the shared address of the first K element (tile base 1024-aligned,
// plus 32 bytes per 8 TF32 K elements).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr)
{
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(16u >> 4) << 16;    // leading byte offset (unused with this swizzle)
    d |= (uint64_t)(1024u >> 4) << 32;  // stride byte offset: 8 rows x 128 bytes
    d |= (uint64_t)1 << 46;             // descriptor version (fixed 0b001)
    d |= (uint64_t)2 << 61;             // swizzle: 128 bytes
    return d;
}

// Instruction descriptor: D f32, A and B tf32, both K-major, M x N.
__host__ __device__ constexpr uint32_t tf32_idesc(int M, int N)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

// FP32 value -> (hi, lo) TF32 pair: hi keeps the top 10 mantissa bits, lo the rest (exact).
__device__ __forceinline__ void split_tf32(float v, float &hi, float &lo)
{
    hi = __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
    lo = __fsub_rn(v, hi);
}

// Byte offset of element (row r, k) in a 128-byte-swizzled K-major tile of
// f32 with 32 K elements per row.
__device__ __forceinline__ uint32_t sw128_off(int r, int k)
{
    return (uint32_t)(r * 128 + ((((k >> 2) ^ (r & 7)) & 7) << 4) + ((k & 3) << 2));
}

// The raw columns and scale of each candidate's source, gathered once per
// call so the kernels read one table entry per candidate instead of following
// the candidate's index arrays for every element: value at row i =
// Src::combine(p0[i * s0], p1[i * s1], prm) (a single load when Src::kRaw is 1).
struct SrcEntry {
    const float *p0;
    const float *p1;
    float prm;
    int s0, s1;
};

template <class Src>
__global__ void k_tc_srctab(Src src, int P, SrcEntry *__restrict__ tab)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < P) {
        tab[j] = SrcEntry{src.raw0(j), src.raw1(j), src.param(j), (int)src.stride0(),
                          (int)src.stride1()};
    }
}

template <class Src>
__device__ __forceinline__ float src_value(const SrcEntry &e, int i)
{
    return Src::kRaw == 2
               ? Src::combine(e.p0[(size_t)i * e.s0], e.p1[(size_t)i * e.s1], e.prm)
               : e.p0[(size_t)i * e.s0];
}

// ---------------------------------------------------------------------------
// Split copies of basis column c.
// ---------------------------------------------------------------------------
__global__ void k_tc_store_column(const float *__restrict__ col, int n, int c,
                                  float *__restrict__ hiC, float *__restrict__ loC, size_t ldn,
                                  float *__restrict__ hiR, float *__restrict__ loR, size_t ldk)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float h, l;
        split_tf32(col[i], h, l);
        hiC[(size_t)c * ldn + i] = h;
        loC[(size_t)c * ldn + i] = l;
        hiR[(size_t)i * ldk + c] = h;
        loR[(size_t)i * ldk + c] = l;
    }
}

// ---------------------------------------------------------------------------
// k_tc_tgemm: Tp[split][j][c] = sum over the split's rows i of src(i, j) Bo[i, c]
//
// The tensor cores add into their FP32 accumulator with truncation, so a long
// accumulation drifts low by about half an ulp per MMA. The sum therefore runs
// in tensor memory over one chunk of TG_CHUNK K steps (128 rows) at a time, in
// two accumulators -- hi*hi, and the small hi*lo + lo*hi -- and drain warps
// add each chunk's sums into FP32 registers (round to nearest) while the MMAs
// of the next chunk fill the other pair of accumulators.
// ---------------------------------------------------------------------------
constexpr int TG_PROD = 8;                                // producer warps
constexpr int TG_DRAIN = 8;                               // drain warps
constexpr int TG_THREADS = 32 * (TG_PROD + 2 + TG_DRAIN);  // + TMA warp + MMA warp
constexpr int TG_M = 128;                                 // candidates per tile
constexpr int TG_K = 32;                                  // rows per K step
constexpr int TG_CHUNK = 4;                               // K steps per accumulation
constexpr int TG_WTMA = TG_PROD, TG_WMMA = TG_PROD + 1, TG_WDRAIN = TG_PROD + 2;

struct TgLayout {
    int S, Np;
    uint32_t a_bytes, b_bytes, stage, bars, total;
    __host__ __device__ TgLayout(int m, int stages)
    {
        S = stages;
        Np = ((m < 16 ? 16 : m) + 15) / 16 * 16;
        a_bytes = TG_M * 128;             // one 128 x 32 f32 operand tile
        b_bytes = (uint32_t)Np * 128;     // one Np x 32 f32 operand tile
        stage = 2 * a_bytes + 2 * b_bytes;  // a_hi, a_lo, b_hi, b_lo
        bars = (uint32_t)S * stage;
        tab = bars + (uint32_t)(3 * S + 5) * 8 + 16;
        total = tab + TG_M * (uint32_t)sizeof(SrcEntry);
    }
    uint32_t tab;
};

// Two loads of 8 consecutive columns of this warp's lanes, one wait.
__device__ __forceinline__ void tmem_ld8x2(uint32_t ta, uint32_t tb, float (&a)[8], float (&b)[8])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%16];\n"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8, %9, %10, %11, %12, %13, %14, %15}, [%17];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(ta), "r"(tb));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        a[i] = __uint_as_float(r[i]);
        b[i] = __uint_as_float(r[8 + i]);
    }
}

template <class Src>
__global__ void __launch_bounds__(TG_THREADS, 1)
    k_tc_tgemm(const SrcEntry *__restrict__ tab, const __grid_constant__ CUtensorMap map_hi,
               const __grid_constant__ CUtensorMap map_lo, int n, int m, int P, int rps,
               int stages, float *__restrict__ Tp, int *__restrict__ err)
{
    extern __shared__ unsigned char smraw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    const TgLayout L(m, stages);
    const int S = L.S, Np = L.Np;
    uint64_t *prod_full = reinterpret_cast<uint64_t *>(sm + L.bars);  // [S] producer warps
    uint64_t *tma_full = prod_full + S;                               // [S] TMA bytes
    uint64_t *empty = tma_full + S;                                   // [S] MMA commit
    uint64_t *acc_full = empty + S;                                   // [2] MMA commit
    uint64_t *acc_empty = acc_full + 2;                               // [2] drain warps
    uint64_t *drain_bar = acc_empty + 2;                              // MMAs in flight at an abort
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain_bar + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    SrcEntry *stab = reinterpret_cast<SrcEntry *>(sm + L.tab);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j0 = blockIdx.x * TG_M, split = blockIdx.y;
    if (threadIdx.x < TG_M) {
        const int j = j0 + threadIdx.x;
        stab[threadIdx.x] = j < P ? tab[j] : SrcEntry{nullptr, nullptr, 0.f, 0, 0};
    }
    const int r0 = split * rps, r1 = min(n, r0 + rps);
    const int ksteps = r1 > r0 ? (r1 - r0 + TG_K - 1) / TG_K : 0;
    const int nchunks = (ksteps + TG_CHUNK - 1) / TG_CHUNK;
    // two buffers x (hi*hi, correction) x Np columns
    const uint32_t ncols = 4 * Np <= 64 ? 64 : 4 * Np <= 128 ? 128 : 4 * Np <= 256 ? 256 : 512;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&prod_full[s], TG_PROD);
            mbar_init(&tma_full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], TG_DRAIN);
        }
        mbar_init(drain_bar, 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == TG_WMMA) {
        tmem_alloc(tmem_slot, ncols);
    }
    if (warp == TG_WTMA && lane == 0) {
        tma_prefetch_desc(&map_hi);
        tma_prefetch_desc(&map_lo);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp < TG_PROD) {
        // Producers: warp w forms rows [4 w, 4 w + 4) of the K step, lane =
        // candidate (lane + 32 q): with row-major sources a warp's loads for
        // one row are contiguous. The loads of step k + 1 are issued before
        // step k is stored, so two steps of source values are in flight.
        float vn[16];
        SrcEntry es[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            es[q] = stab[lane + 32 * q];
        }
        auto load = [&](int k) {
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
                const int i = r0 + k * TG_K + 4 * warp + rr;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    vn[4 * rr + q] =
                        (i < r1 && es[q].p0 != nullptr) ? src_value<Src>(es[q], i) : 0.f;
                }
            }
        };
        if (ksteps > 0) {
            load(0);
        }
        for (int k = 0; k < ksteps; ++k) {
            const int s = k % S, fill = k / S;
            float v[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                v[q] = vn[q];
            }
            if (k + 1 < ksteps) {
                load(k + 1);
            }
            if (fill >= 1 && !mbar_wait_warp(&empty[s], (fill - 1) & 1, abort_flag, err)) {
                break;
            }
            unsigned char *ahi = sm + (size_t)s * L.stage;
            unsigned char *alo = ahi + L.a_bytes;
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    float h, l;
                    split_tf32(v[4 * rr + q], h, l);
                    const uint32_t off = sw128_off(lane + 32 * q, 4 * warp + rr);
                    *reinterpret_cast<float *>(ahi + off) = h;
                    *reinterpret_cast<float *>(alo + off) = l;
                }
            }
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&prod_full[s]);
            }
        }
    } else if (warp == TG_WTMA) {
        // TMA: the Bo rows of each K step, hi and lo.
        if (lane == 0) {
            int issued = 0;
            for (int k = 0; k < ksteps; ++k) {
                const int s = k % S, fill = k / S;
                if (fill >= 1 && !mbar_wait(&empty[s], (fill - 1) & 1, abort_flag, err)) {
                    break;
                }
                unsigned char *bhi = sm + (size_t)s * L.stage + 2 * L.a_bytes;
                unsigned char *blo = bhi + L.b_bytes;
                mbar_expect_tx(&tma_full[s], 2 * L.b_bytes);
                const int x = r0 + k * TG_K;
                tma_load_2d(bhi, &map_hi, x, 0, &tma_full[s]);
                tma_load_2d(blo, &map_lo, x, 0, &tma_full[s]);
                issued = k + 1;
            }
            // let every copy issued land before the block can exit
            for (int k = issued > S ? issued - S : 0; k < issued; ++k) {
                mbar_wait(&tma_full[k % S], (k / S) & 1, abort_flag, err, true);
            }
        }
    } else if (warp == TG_WMMA) {
        // MMA issuer: chunk q accumulates into buffer q & 1.
        if (lane == 0) {
            const uint32_t idesc = tf32_idesc(TG_M, Np);
            bool ok = true;
            for (int q = 0; q < nchunks && ok; ++q) {
                const int b = q & 1;
                if (q >= 2 && !mbar_wait(&acc_empty[b], ((q >> 1) - 1) & 1, abort_flag, err)) {
                    break;
                }
                tc_fence_after();
                const uint32_t dmain = tmem + (uint32_t)(b * 2 * Np), dcorr = dmain + Np;
                const int k1 = min(ksteps, (q + 1) * TG_CHUNK);
                for (int k = q * TG_CHUNK; k < k1; ++k) {
                    const int s = k % S, ph = (k / S) & 1;
                    if (!mbar_wait(&prod_full[s], ph, abort_flag, err) ||
                        !mbar_wait(&tma_full[s], ph, abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t base = smem_u32(sm + (size_t)s * L.stage);
                    const uint32_t ahi = base, alo = base + L.a_bytes;
                    const uint32_t bhi = base + 2 * L.a_bytes, blo = bhi + L.b_bytes;
#pragma unroll
                    for (int kk = 0; kk < TG_K / 8; ++kk) {
                        const uint32_t o = 32u * kk;
                        const uint32_t acc = (k > q * TG_CHUNK || kk > 0) ? 1u : 0u;
                        mma_tf32(dmain, sw128_desc(ahi + o), sw128_desc(bhi + o), idesc, acc);
                        mma_tf32(dcorr, sw128_desc(ahi + o), sw128_desc(blo + o), idesc, acc);
                        mma_tf32(dcorr, sw128_desc(alo + o), sw128_desc(bhi + o), idesc, 1u);
                    }
                    mma_commit(&empty[s]);
                }
                if (ok) {
                    mma_commit(&acc_full[b]);
                }
            }
            if (*abort_flag) {
                mma_commit(drain_bar);  // lands once every MMA issued so far has completed
                mbar_wait(drain_bar, 0, abort_flag, err, true);
            }
        }
    } else {
        // Drain warps: lanes 32 (w % 4) .. (candidates), one half of the
        // columns (basis components) each.
        const int g = warp - TG_WDRAIN, lg = warp & 3, h = g >> 2;
        const int nph = Np / 2;  // columns per drain warp, a multiple of 8, <= 64
        float acc[64];
#pragma unroll
        for (int c = 0; c < 64; ++c) {
            acc[c] = 0.f;
        }
        bool ok = true;
        for (int q = 0; q < nchunks; ++q) {
            const int b = q & 1;
            if (!mbar_wait_warp(&acc_full[b], (q >> 1) & 1, abort_flag, err)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t tm = tmem + ((uint32_t)(32 * lg) << 16) +
                                (uint32_t)(b * 2 * Np + h * nph);
#pragma unroll
            for (int c8 = 0; c8 < 8; ++c8) {
                if (8 * c8 < nph) {
                    float x[8], y[8];
                    tmem_ld8x2(tm + 8 * c8, tm + Np + 8 * c8, x, y);
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        acc[8 * c8 + t] = __fadd_rn(acc[8 * c8 + t], __fadd_rn(x[t], y[t]));
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&acc_empty[b]);
            }
        }
        const int j = j0 + 32 * lg + lane;
        if (ok && j < P) {
            float *dst = Tp + ((size_t)split * P + j) * m + h * nph;
#pragma unroll
            for (int c = 0; c < 64; ++c) {
                if (c < nph && h * nph + c < m) {
                    dst[c] = acc[c];
                }
            }
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    if (warp == TG_WMMA) {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
}

// T[j][c] = f32(sum over splits of Tp), in a fixed order, plus the split copies
// Thi/Tlo [P][ldk] (zero past m).
__global__ void k_tc_treduce(const float *__restrict__ Tp, int ks, int P, int m, size_t ldk,
                             float *__restrict__ T, float *__restrict__ Thi,
                             float *__restrict__ Tlo)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)P * ldk) {
        return;
    }
    const int j = (int)(e / ldk), c = (int)(e % ldk);
    float t = 0.f;
    if (c < m) {
        const size_t cnt = (size_t)P * m, idx = (size_t)j * m + c;
        double a = 0.0;
        for (int q = 0; q < ks; ++q) {
            a += (double)Tp[(size_t)q * cnt + idx];
        }
        t = (float)a;
        T[idx] = t;
    }
    float h, l;
    split_tf32(t, h, l);
    Thi[e] = h;
    Tlo[e] = l;
}

// ---------------------------------------------------------------------------
// k_tc_project: Bx[i, j] = src(i, j) - sum_c Bo[i, c] T[j][c], persistent
// ---------------------------------------------------------------------------
constexpr int TP_EPI = 8;                       // epilogue warps
constexpr int TP_THREADS = 32 * (TP_EPI + 2);   // + TMA warp + MMA warp
constexpr int TP_M = 128;                       // rows per tile
constexpr int TP_N = 64;                        // candidates per tile
constexpr int TP_S = 2;                         // K-step stages

struct TpLayout {
    uint32_t a_bytes, b_bytes, stage, bars, total;
    __host__ __device__ TpLayout()
    {
        a_bytes = TP_M * 128;
        b_bytes = TP_N * 128;
        stage = 2 * a_bytes + 2 * b_bytes;
        bars = TP_S * stage;
        total = bars + (2 * TP_S + 5) * 8 + 16;
    }
};

template <class Src>
__global__ void __launch_bounds__(TP_THREADS, 2)
    k_tc_project(const SrcEntry *__restrict__ tab, const __grid_constant__ CUtensorMap a_hi,
                 const __grid_constant__ CUtensorMap a_lo, const __grid_constant__ CUtensorMap b_hi,
                 const __grid_constant__ CUtensorMap b_lo, int n, int m, int P,
                 float *__restrict__ Bx, size_t ldr, int *__restrict__ err)
{
    extern __shared__ unsigned char smraw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    const TpLayout L;
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + L.bars);  // [TP_S] TMA bytes
    uint64_t *empty = full + TP_S;                               // [TP_S] MMA commit
    uint64_t *acc_full = empty + TP_S;                           // [2]
    uint64_t *acc_empty = acc_full + 2;                          // [2] epilogue warps
    uint64_t *drain = acc_empty + 2;                             // MMAs in flight at an abort
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rt = (n + TP_M - 1) / TP_M, ct = (P + TP_N - 1) / TP_N;
    const long tiles = (long)rt * ct;
    const int kt = (m + 31) / 32;
    const uint32_t ncols = 4 * TP_N;  // two buffers x (hi*hi, correction)

    if (threadIdx.x == 0) {
        for (int s = 0; s < TP_S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], TP_EPI);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == TP_EPI + 1) {
        tmem_alloc(tmem_slot, ncols);
    }
    if (warp == TP_EPI && lane == 0) {
        tma_prefetch_desc(&a_hi);
        tma_prefetch_desc(&a_lo);
        tma_prefetch_desc(&b_hi);
        tma_prefetch_desc(&b_lo);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // tile t: candidate tile t % ct (fastest), row tile t / ct
    if (warp == TP_EPI) {
        if (lane == 0) {
            long g = 0, issued = 0;
            bool ok = true;
            for (long t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
                const int row0 = (int)(t / ct) * TP_M, cand0 = (int)(t % ct) * TP_N;
                for (int k = 0; k < kt; ++k, ++g) {
                    const int s = (int)(g % TP_S);
                    const long fill = g / TP_S;
                    if (fill >= 1 && !mbar_wait(&empty[s], (uint32_t)((fill - 1) & 1), abort_flag,
                                                err)) {
                        ok = false;
                        break;
                    }
                    unsigned char *st = sm + (size_t)s * L.stage;
                    mbar_expect_tx(&full[s], L.stage);
                    tma_load_2d(st, &a_hi, 32 * k, row0, &full[s]);
                    tma_load_2d(st + L.a_bytes, &a_lo, 32 * k, row0, &full[s]);
                    tma_load_2d(st + 2 * L.a_bytes, &b_hi, 32 * k, cand0, &full[s]);
                    tma_load_2d(st + 2 * L.a_bytes + L.b_bytes, &b_lo, 32 * k, cand0, &full[s]);
                    issued = g + 1;
                }
            }
            for (long q = issued > TP_S ? issued - TP_S : 0; q < issued; ++q) {
                mbar_wait(&full[q % TP_S], (uint32_t)((q / TP_S) & 1), abort_flag, err, true);
            }
        }
    } else if (warp == TP_EPI + 1) {
        if (lane == 0) {
            const uint32_t idesc = tf32_idesc(TP_M, TP_N);
            long g = 0, u = 0;
            bool ok = true;
            for (long t = blockIdx.x; t < tiles && ok; t += gridDim.x, ++u) {
                const int b = (int)(u & 1);
                if (u >= 2 && !mbar_wait(&acc_empty[b], (uint32_t)(((u >> 1) - 1) & 1),
                                         abort_flag, err)) {
                    break;
                }
                tc_fence_after();
                const uint32_t dmain = tmem + (uint32_t)(b * 2 * TP_N), dcorr = dmain + TP_N;
                for (int k = 0; k < kt; ++k, ++g) {
                    const int s = (int)(g % TP_S);
                    if (!mbar_wait(&full[s], (uint32_t)((g / TP_S) & 1), abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t base = smem_u32(sm + (size_t)s * L.stage);
                    const uint32_t ahi = base, alo = base + L.a_bytes;
                    const uint32_t bhi = base + 2 * L.a_bytes, blo = bhi + L.b_bytes;
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk) {
                        const uint32_t o = 32u * kk;
                        const uint32_t acc = (k > 0 || kk > 0) ? 1u : 0u;
                        mma_tf32(dmain, sw128_desc(ahi + o), sw128_desc(bhi + o), idesc, acc);
                        mma_tf32(dcorr, sw128_desc(ahi + o), sw128_desc(blo + o), idesc, acc);
                        mma_tf32(dcorr, sw128_desc(alo + o), sw128_desc(bhi + o), idesc, 1u);
                    }
                    mma_commit(&empty[s]);
                }
                if (ok) {
                    mma_commit(&acc_full[b]);
                }
            }
            if (*abort_flag) {
                mma_commit(drain);  // lands once every MMA issued so far has completed
                mbar_wait(drain, 0, abort_flag, err, true);
            }
        }
    } else {
        // Epilogue: warp w reads lanes 32 (w % 4) .. (the tile's rows) and
        // handles candidates [32 h, 32 h + 32), h = w / 4, in two groups of
        // 16: the source values are loaded before the accumulator is waited
        // for, so their latency overlaps the MMAs.
        const int lg = warp & 3, h = warp >> 2;
        long u = 0;
        bool ok = true;
        for (long t = blockIdx.x; t < tiles && ok; t += gridDim.x, ++u) {
            const int b = (int)(u & 1);
            const int row0 = (int)(t / ct) * TP_M, cand0 = (int)(t % ct) * TP_N + 32 * h;
            const int i = row0 + 32 * lg + lane;
            for (int g = 0; g < 2; ++g) {
                float v[16];
                const int jg = cand0 + 16 * g;  // a multiple of 16
                if (Src::kRaw == 1) {
                    // row-major stored columns: four 16-byte loads of this row
                    // (rows are 16-byte aligned; the padding up to a multiple
                    // of 4 candidates is in bounds)
                    const float *row = tab[0].p0 + (size_t)i * tab[0].s0;
#pragma unroll
                    for (int k4 = 0; k4 < 4; ++k4) {
                        const int j = jg + 4 * k4;
                        const float4 w = (i < n && j < P)
                                             ? *reinterpret_cast<const float4 *>(row + j)
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
                        v[4 * k4] = w.x;
                        v[4 * k4 + 1] = w.y;
                        v[4 * k4 + 2] = w.z;
                        v[4 * k4 + 3] = w.w;
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const int j = jg + q;
                        v[q] = (i < n && j < P) ? src_value<Src>(tab[j], i) : 0.f;
                    }
                }
                if (g == 0) {
                    if (!mbar_wait_warp(&acc_full[b], (uint32_t)((u >> 1) & 1), abort_flag, err)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                }
                const uint32_t tm = tmem + ((uint32_t)(32 * lg) << 16) +
                                    (uint32_t)(b * 2 * TP_N + 32 * h + 16 * g);
                float x0[8], y0[8], x1[8], y1[8];
                tmem_ld8x2(tm, tm + TP_N, x0, y0);
                tmem_ld8x2(tm + 8, tm + TP_N + 8, x1, y1);
                if (i < n) {
                    float o[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const float d = q < 8 ? __fadd_rn(x0[q], y0[q])
                                              : __fadd_rn(x1[q - 8], y1[q - 8]);
                        o[q] = __fsub_rn(v[q], d);
                    }
                    // 16-byte stores; columns past P up to ldr are padding
                    float *row = Bx + (size_t)i * ldr;
#pragma unroll
                    for (int k4 = 0; k4 < 4; ++k4) {
                        const int j = jg + 4 * k4;
                        if (j < P) {
                            *reinterpret_cast<float4 *>(row + j) =
                                make_float4(o[4 * k4], o[4 * k4 + 1], o[4 * k4 + 2], o[4 * k4 + 3]);
                        }
                    }
                }
            }
            if (!ok) {
                break;
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&acc_empty[b]);
            }
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    if (warp == TP_EPI + 1) {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                 const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                 const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_tiled()
{
    static std::once_flag once;
    static EncodeTiled fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess) {
            fn = reinterpret_cast<EncodeTiled>(p);
        }
    });
    verify(fn != nullptr, "cuTensorMapEncodeTiled is not available from the driver", 2);
    return fn;
}

// 2-D f32 tensor map: `inner` contiguous elements per line, `outer` lines,
// `pitch` elements between lines; box 32 x box_outer, 128-byte swizzle.
CUtensorMap tmap_2d(const float *base, size_t inner, size_t outer, size_t pitch,
                    uint32_t box_outer)
{
    verify(reinterpret_cast<uintptr_t>(base) % 16 == 0 && pitch % 4 == 0,
           "tensor map base or pitch not 16-byte aligned", 2);
    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(float)};
    const cuuint32_t box[2] = {32u, box_outer};
    const cuuint32_t es[2] = {1u, 1u};
    const CUresult r = encode_tiled()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                      const_cast<float *>(base), dims, strides, box, es,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        throw Error(2, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    }
    return map;
}

int sm_count()
{
    int dev = 0, c = 0;
    CUDA_CHECK(cudaGetDevice(&dev));
    CUDA_CHECK(cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev));
    return std::max(1, c);
}

int tg_stages(int m)
{
    const size_t budget = 220 * 1024;
    for (int S = 4; S >= 2; --S) {
        if (TgLayout(m, S).total + 1024 <= budget) {
            return S;
        }
    }
    return 2;
}

void check_err(cudaStream_t st, int *err)
{
    int h = 0;
    CUDA_CHECK(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_CHECK(cudaStreamSynchronize(st));
    verify(h == 0, "a bounded wait in the tensor-core projection ran out", MARS_GPU_ETIMEOUT);
}

template <class Src>
void build_tab(cudaStream_t st, const Src &src, int P, SrcEntry *tab, long long *launches)
{
    k_tc_srctab<Src><<<(unsigned)ceil_div((size_t)P, 256), 256, 0, st>>>(src, P, tab);
    LAUNCH_CHECK();
    *launches += 1;
}

template <class Src>
void t_pass(cudaStream_t st, const Src &src, const TcBasis &tb, int n, int m, int P,
            const TcScratch &ws, long long *launches)
{
    const int ks = tc_ksplit(n, P);
    const int rps = (int)round_up(ceil_div((size_t)n, (size_t)ks), TG_K);
    const int S = tg_stages(m);
    const TgLayout L(m, S);
    const CUtensorMap mh = tmap_2d(tb.hiC, tb.ldn, (size_t)m, tb.ldn, (uint32_t)L.Np);
    const CUtensorMap ml = tmap_2d(tb.loC, tb.ldn, (size_t)m, tb.ldn, (uint32_t)L.Np);
    const size_t smem = L.total + 1024;
    allow_smem(k_tc_tgemm<Src>, smem);
    const dim3 grid((unsigned)ceil_div((size_t)P, TG_M), (unsigned)ks);
    k_tc_tgemm<Src><<<grid, TG_THREADS, smem, st>>>(static_cast<const SrcEntry *>(ws.tab), mh, ml, n, m, P, rps, S, ws.Tp,
                                                     ws.err);
    LAUNCH_CHECK();
    const size_t cnt = (size_t)P * tb.ldk;
    k_tc_treduce<<<(unsigned)ceil_div(cnt, 256), 256, 0, st>>>(ws.Tp, ks, P, m, tb.ldk, ws.T,
                                                              ws.Thi, ws.Tlo);
    LAUNCH_CHECK();
    *launches += 2;
}

template <class Src>
void p_pass(cudaStream_t st, const Src &src, const TcBasis &tb, int n, int m, int P,
            const TcScratch &ws, long long *launches)
{
    const CUtensorMap ah = tmap_2d(tb.hiR, tb.ldk, (size_t)n, tb.ldk, TP_M);
    const CUtensorMap al = tmap_2d(tb.loR, tb.ldk, (size_t)n, tb.ldk, TP_M);
    const CUtensorMap bh = tmap_2d(ws.Thi, tb.ldk, (size_t)P, tb.ldk, TP_N);
    const CUtensorMap bl = tmap_2d(ws.Tlo, tb.ldk, (size_t)P, tb.ldk, TP_N);
    const TpLayout L;
    const size_t smem = L.total + 1024;
    allow_smem(k_tc_project<Src>, smem);
    const long tiles = (long)ceil_div((size_t)n, TP_M) * (long)ceil_div((size_t)P, TP_N);
    const long grid = std::min<long>(tiles, 2L * sm_count());
    k_tc_project<Src><<<(unsigned)grid, TP_THREADS, smem, st>>>(static_cast<const SrcEntry *>(ws.tab), ah, al, bh, bl, n, m,
                                                                P, ws.Bx, ws.ldr, ws.err);
    LAUNCH_CHECK();
    *launches += 1;
}

}  // namespace

size_t tc_ldn(size_t n) { return round_up(std::max<size_t>(n, 1), 32); }
size_t tc_tab_bytes(size_t P) { return sizeof(SrcEntry) * std::max<size_t>(P, 1); }
size_t tc_ldk(size_t max_terms) { return round_up(std::max<size_t>(max_terms, 1), 32); }

void tc_store_column(cudaStream_t st, const float *col, int n, int c, const TcBasis &tb,
                     long long *launches)
{
    k_tc_store_column<<<(unsigned)ceil_div((size_t)n, 256), 256, 0, st>>>(
        col, n, c, tb.hiC, tb.loC, tb.ldn, tb.hiR, tb.loR, tb.ldk);
    LAUNCH_CHECK();
    *launches += 1;
}

int tc_ksplit(int n, int P)
{
    // one wave of one block per SM (a second, partial wave would double the time)
    const int tiles = (int)ceil_div((size_t)std::max(P, 1), TG_M);
    const int want = std::max(1, sm_count() / tiles);
    return std::max(1, std::min(want, std::max(1, n / (8 * TG_K))));
}

void tc_project_pass(cudaStream_t st, const RowFillSrc &src, const TcBasis &tb, int n, int m,
                     int P, const TcScratch &ws, long long *launches)
{
    verify(m >= 1 && m <= TC_MAX_M, "the tensor-core projection takes 1..128 basis columns");
    CUDA_CHECK(cudaMemsetAsync(ws.err, 0, sizeof(int), st));
    build_tab(st, src, P, static_cast<SrcEntry *>(ws.tab), launches);
    t_pass(st, src, tb, n, m, P, ws, launches);
    p_pass(st, src, tb, n, m, P, ws, launches);
    check_err(st, ws.err);
}

void fast_project_tc(cudaStream_t st, const FillSrc &src, const RowFillSrc &rsrc,
                     const TcBasis &tb, int n, int m, int P, const float *y, double tol,
                     const TcScratch &ws, long long *launches)
{
    if (P <= 0) {
        return;
    }
    verify(m >= 1 && m <= TC_MAX_M, "the tensor-core projection takes 1..128 basis columns");
    CUDA_CHECK(cudaMemsetAsync(ws.err, 0, sizeof(int), st));
    build_tab(st, rsrc, P, static_cast<SrcEntry *>(ws.tab), launches);
    t_pass(st, rsrc, tb, n, m, P, ws, launches);
    p_pass(st, rsrc, tb, n, m, P, ws, launches);
    const RowStoredSrc stored{ws.Bx, ws.ldr};
    build_tab(st, stored, P, static_cast<SrcEntry *>(ws.tab), launches);
    t_pass(st, stored, tb, n, m, P, ws, launches);
    p_pass(st, stored, tb, n, m, P, ws, launches);
    fast_norms_rows(st, ws.Bx, ws.ldr, n, y, tol, P, ws.npart, ws.s, ws.ybx, launches);
    fast_parent_moments(st, src, n, P, ws.mom, launches);
    check_err(st, ws.err);
}

}  // namespace mgpu

// ===========================================================================
// Kernel-level entry point (host arrays), for tests and micro-benchmarks.
// ===========================================================================
extern "C" {

MARS_GPU_API int mars_gpu_fast_project(size_t n, size_t m, size_t P, const float *B, size_t ldB,
                                       size_t ncolB, const float *X, size_t ldX, size_t ncolX,
                                       const float *s, const int *cand_x, const int *cand_b,
                                       const float *Bo, size_t ldBo, const float *y, double tol,
                                       int use_tc, int passes, float *T, float *Bx,
                                       double *s_out, double *ybx_out, float *ms_out)
{
    using namespace mgpu;
    try {
        verify(B && X && s && cand_x && cand_b && Bo && y && T && Bx, "null argument");
        verify(n >= 1 && m >= 1 && P >= 1 && n <= 0x7fffffff && P <= 0x7fffffff,
               "empty or oversized problem");
        verify(ldB >= n && ldX >= n && ldBo >= n, "leading dimension smaller than the data");
        verify(passes == 1 || passes == 2, "passes must be 1 or 2");
        verify(use_tc || passes == 2, "the FP32 SIMT projection runs both passes");
        for (size_t j = 0; j < P; ++j) {
            verify(cand_x[j] >= 0 && (size_t)cand_x[j] < ncolX &&
                       cand_b[j] >= 0 && (size_t)cand_b[j] < ncolB,
                   "candidate index outside the columns of X or B");
        }
        if (use_tc) {
            verify(m <= (size_t)TC_MAX_M, "the tensor-core projection takes 1..128 basis columns");
        }
        cudaStream_t st = nullptr;
        CUDA_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
        } guard{st};
        DevBuf dB, dX, ds, dcx, dcb, dBoC, dy, dTp, dT, dThi, dTlo, dBx, dS, dYbx, dMom, dErr,
            hiC, loC, hiR, loR, dTab, dBR, dNpart, dBxc;
        for (DevBuf *b : {&dB, &dX, &ds, &dcx, &dcb, &dBoC, &dy, &dTp, &dT, &dThi, &dTlo, &dBx,
                          &dS, &dYbx, &dMom, &dErr, &hiC, &loC, &hiR, &loR, &dTab, &dBR, &dNpart,
                          &dBxc}) {
            b->bind(st);
        }
        dB.ensure(sizeof(float) * n * ncolB);
        CUDA_CHECK(cudaMemcpy2DAsync(dB.ptr, n * 4, B, ldB * 4, n * 4, ncolB,
                                     cudaMemcpyHostToDevice, st));
        dX.ensure(sizeof(float) * n * ncolX);
        CUDA_CHECK(cudaMemcpy2DAsync(dX.ptr, n * 4, X, ldX * 4, n * 4, ncolX,
                                     cudaMemcpyHostToDevice, st));
        ds.ensure(sizeof(float) * ncolX);
        CUDA_CHECK(cudaMemcpyAsync(ds.ptr, s, sizeof(float) * ncolX, cudaMemcpyHostToDevice, st));
        dcx.ensure(sizeof(int) * P);
        dcb.ensure(sizeof(int) * P);
        CUDA_CHECK(cudaMemcpyAsync(dcx.ptr, cand_x, sizeof(int) * P, cudaMemcpyHostToDevice, st));
        CUDA_CHECK(cudaMemcpyAsync(dcb.ptr, cand_b, sizeof(int) * P, cudaMemcpyHostToDevice, st));
        dBoC.ensure(sizeof(float) * n * m);
        CUDA_CHECK(cudaMemcpy2DAsync(dBoC.ptr, n * 4, Bo, ldBo * 4, n * 4, m,
                                     cudaMemcpyHostToDevice, st));
        dy.ensure(sizeof(float) * n);
        CUDA_CHECK(cudaMemcpyAsync(dy.ptr, y, sizeof(float) * n, cudaMemcpyHostToDevice, st));
        const size_t ldr = round_up(P, 4), ldbr = round_up(ncolB, 4);
        dBx.ensure(sizeof(float) * n * ldr);
        dBR.ensure(sizeof(float) * n * ldbr);
        dS.ensure(sizeof(double) * P);
        dYbx.ensure(sizeof(double) * P);
        dMom.ensure(sizeof(double) * 3 * P);
        dT.ensure(sizeof(float) * P * m);
        long long launches = 0;
        const FillSrc src{dB.as<float>(), n, dX.as<float>(), n, ds.as<float>(), dcx.as<int>(),
                          dcb.as<int>()};
        fast_to_rows(st, dB.as<float>(), (int)n, (int)ncolB, dBR.as<float>(), ldbr, &launches);
        const RowFillSrc rsrc{dBR.as<float>(), ldbr, dX.as<float>(), n, ds.as<float>(),
                              dcx.as<int>(), dcb.as<int>()};
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        CUDA_CHECK(cudaEventCreate(&e0));
        CUDA_CHECK(cudaEventCreate(&e1));
        struct EventGuard {
            cudaEvent_t a, b;
            ~EventGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
        } eguard{e0, e1};
        if (use_tc) {
            TcBasis tb;
            tb.ldn = tc_ldn(n);
            tb.ldk = tc_ldk(m);
            hiC.ensure(sizeof(float) * tb.ldn * m);
            loC.ensure(sizeof(float) * tb.ldn * m);
            hiR.ensure(sizeof(float) * n * tb.ldk);
            loR.ensure(sizeof(float) * n * tb.ldk);
            for (DevBuf *b : {&hiC, &loC, &hiR, &loR}) {
                CUDA_CHECK(cudaMemsetAsync(b->ptr, 0, b->bytes, st));
            }
            tb.hiC = hiC.as<float>();
            tb.loC = loC.as<float>();
            tb.hiR = hiR.as<float>();
            tb.loR = loR.as<float>();
            for (size_t c = 0; c < m; ++c) {
                tc_store_column(st, dBoC.as<float>() + c * n, (int)n, (int)c, tb, &launches);
            }
            const int ks = tc_ksplit((int)n, (int)P);
            dTp.ensure(sizeof(float) * (size_t)ks * P * m);
            dThi.ensure(sizeof(float) * P * tb.ldk);
            dTlo.ensure(sizeof(float) * P * tb.ldk);
            dErr.ensure(sizeof(int));
            dTab.ensure(tc_tab_bytes(P));
            dNpart.ensure(fast_norm_part_bytes(n, P));
            TcScratch ws{dTp.as<float>(), dT.as<float>(),    dThi.as<float>(),
                         dTlo.as<float>(), dBx.as<float>(),  ldr,
                         dS.as<double>(),  dYbx.as<double>(), dMom.as<double>(),
                         dErr.as<int>(),   dTab.ptr,          dNpart.as<double>()};
            CUDA_CHECK(cudaEventRecord(e0, st));
            if (passes == 1) {
                tc_project_pass(st, rsrc, tb, (int)n, (int)m, (int)P, ws, &launches);
            } else {
                fast_project_tc(st, src, rsrc, tb, (int)n, (int)m, (int)P, dy.as<float>(), tol,
                                ws, &launches);
            }
        } else {
            const int ks = fast_ksplit((int)n);
            dTp.ensure(sizeof(float) * (size_t)ks * P * m);
            dBxc.ensure(sizeof(float) * n * P);
            FastScratch ws{dTp.as<float>(), dT.as<float>(), dBxc.as<float>(), dS.as<double>(),
                           dYbx.as<double>(), dMom.as<double>()};
            CUDA_CHECK(cudaEventRecord(e0, st));
            fast_project(st, src, dBoC.as<float>(), (int)n, (int)m, (int)P, dy.as<float>(), tol,
                         ws, &launches);
            fast_to_rows(st, dBxc.as<float>(), (int)n, (int)P, dBx.as<float>(), ldr, &launches);
        }
        CUDA_CHECK(cudaEventRecord(e1, st));
        CUDA_CHECK(cudaMemcpyAsync(T, dT.ptr, sizeof(float) * P * m, cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaMemcpy2DAsync(Bx, P * 4, dBx.ptr, ldr * 4, P * 4, n,
                                     cudaMemcpyDeviceToHost, st));
        if (s_out && passes == 2) {
            CUDA_CHECK(cudaMemcpyAsync(s_out, dS.ptr, sizeof(double) * P, cudaMemcpyDeviceToHost,
                                       st));
        }
        if (ybx_out && passes == 2) {
            CUDA_CHECK(cudaMemcpyAsync(ybx_out, dYbx.ptr, sizeof(double) * P,
                                       cudaMemcpyDeviceToHost, st));
        }
        CUDA_CHECK(cudaStreamSynchronize(st));
        if (ms_out) {
            CUDA_CHECK(cudaEventElapsedTime(ms_out, e0, e1));
        }
        return MARS_GPU_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.status;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return MARS_GPU_ECUDA;
    }
}

}  // extern "C"
