// The exact append on the GPU (marsalgo.cc:760-875 MarsAlgo::append,
// kernels.cc:194-281 orthonormalize_col): the new column from its input and
// parent, its raw norm, the modified Gram-Schmidt chains against the basis
// (with the DGKS re-pass), the norm of the result and its dot with y. Each is a
// sequential FP64 fused-multiply-add chain over the rows in order, and each is
// evaluated exactly in parallel (xchain.cuh) by one launch over the whole GPU:
//
//   1. every thread owns a chunk of L consecutive rows; it applies the row
//      operations that lead to the chain's terms (the column build, the update
//      v <- fma(-c, q, v) with the previous chain's value, the normalisation)
//      and sums the chain's terms in float-float;
//   2. a block scan of those sums, on top of the block's entry guess, guesses
//      each chunk's entry value; the chunk runs the chain speculatively from it
//      (XcSpecR) and leaves a record;
//   3. the records compose level by level (8 chunks, 4 sub-groups of a warp, 8
//      warps of a block) into one record per block, which carries 8 residues
//      where the lower levels carry 4;
//   4. the last block to finish (a ticket, no waiting) composes the blocks in
//      groups of 16, walks the groups from the true start 0 -- descending into
//      the sub-records, down to re-running rows, wherever a record cannot vouch
//      for its entry -- and stores the chain's value; it also turns the blocks'
//      aggregates of the next chain's terms (polynomials in this chain's
//      value) into the next launch's block entry guesses.
// The value is the sequential chain's bit for bit whatever the data; the
// guesses only decide how much is re-run.
#include "xappend.cuh"
#include "xchain.cuh"

#include <algorithm>
#include <cmath>

namespace mgpu {
namespace {

constexpr int XA_T = 256;             // threads (one chunk each) per block
constexpr int XA_NW = XA_T / 32;      // warps per block
constexpr int XA_SUB = 8;             // chunks per sub-group
constexpr int XA_NS = XA_T / XA_SUB;  // sub-groups per block (4 per warp)
constexpr int XA_GRP = 16;            // blocks per group of the final walk
constexpr int XA_MAXG = XA_T;         // blocks per launch at most
constexpr int XA_LMIN = 8;            // rows per chunk at least, below XA_MAXG blocks
constexpr int XA_TILE = 8;            // rows whose loads a thread issues together
constexpr long long XA_MAX_CHAINS = 65535;  // side-by-side chains per launch (grid y)
constexpr size_t XA_REC_BUDGET = 1ull << 30;  // bytes of records for side-by-side chains
constexpr int XA_LANES = XC_RUNS + 1;
// Block and group records carry more residues than the chunks': a walk from the
// true start crosses them where a 4-residue record, allowed one binade of rise
// above its start, would send it down into the block's sub-records.
constexpr int XA_RB = 8;
constexpr int XA_LANES_B = XA_RB + 1;
using XcRecB = XcRecT<XA_RB>;
// bytes of dynamic shared memory for a block's own records, which the last
// block reuses for the blocks' records
constexpr size_t XA_SMEM_OWN =
    (std::max(sizeof(XcRec) * (XA_T + XA_NS + XA_NW), sizeof(XcRecB) * XA_MAXG) + 15) / 16 * 16;

// result slots
constexpr int R_RAW2 = 0, R_VN = 1, R_VN2 = 2, R_YBO = 3, R_C = 4;

enum : int { XA_NONE = 0, XA_SQ, XA_QV, XA_QY };  // chain terms: v v, q v, q y
enum : int {  // aggregates of the next chain's terms, as polynomials a0 + a1 c + a2 c^2
    XN_NONE = 0,
    XN_SQ,      // v v
    XN_QV,      // q_next v
    XN_QY,      // (stored f32 column) y
    XN_QV_UPD,  // q_next (v - c q):  a0 = q_next v, a1 = -q_next q
    XN_SQ_UPD,  // (v - c q)^2:       a0 = v v, a1 = -2 v q, a2 = q q
    XN_AB,      // q y: the terms of this launch's own XA_QY chains (their guesses)
};

struct XaArgs {
    int n, L;
    // row operations, in this order
    int fill;  // B[:, mcol] = the new column from X[:, xcol] and B[:, bcol]; v_out = it
    char type;
    const float *X;
    size_t ldX;
    const float *s;
    int xcol, bcol;
    float h;
    int scale;  // B[:, mcol] /= f32(sqrt(res[R_RAW2]))
    float *B;   // column-major, column stride n (fill, scale)
    int upd;    // v_out = fma(-res[c_slot], q_prev, v_in)
    const float *q_prev;
    int c_slot;
    int norm;  // v = v_in / sqrt(res[w_slot]); q_out = f32(v) (when given)
    int w_slot;
    float *q_out;
    int mcol;
    const double *v_in;
    double *v_out;
    // this launch's chain
    int kind;
    const float *q;
    const float *y;
    int res_slot;
    // the next chain's aggregates
    int next;
    const float *q_next;
    const double *g_in;  // this chain's block entry guesses
    double *g_out;       // the next chain's
    // Independent chains side by side, blockIdx.y = chain c (one chain: c = 0):
    // its q column q + (c % qk) qld, its y column y + ycol[c / qk] yld (ycol
    // null: c / qk), and its records, aggregates, guesses, ticket and result
    // (res[res_slot + c]) at per-chain offsets.
    int qk;
    size_t qld, yld;
    const int *ycol;
    // scratch
    double *res;
    XcRec *rc, *rs, *rw;
    XcRecB *rb;
    double *agg;
    unsigned *ticket;
};

// GB300 runs conversions to and from f64 on its narrow FP64 pipe, which the
// chains' fused multiply-adds already keep busy: xc_f2d (xchain.cuh) and this
// build the values from their bit fields on the integer pipe instead.

// An approximate float-float split of an f64 (for guesses only): h its
// leading 24 significant bits, l most of the rest; 0 where the value is
// outside the normal float range.
__device__ __forceinline__ void ff_of(double v, float &h, float &l)
{
    const uint32_t hi = (uint32_t)__double2hiint(v), lo = (uint32_t)__double2loint(v);
    const int E = (int)((hi >> 20) & 0x7ffu);
    if (E < 1023 - 70 || E > 1023 + 100) {
        h = 0.0f;
        l = 0.0f;
        return;
    }
    const uint32_t sgn = hi & 0x80000000u;
    h = __uint_as_float(sgn | ((uint32_t)(E - 896) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
    const float r = __uint2float_rn(lo & 0x1fffffffu);            // the low 29 bits, in units of
    const float scale = __uint_as_float((uint32_t)(E - 1075 + 127) << 23);  // 2^(E - 1075)
    l = sgn ? -(r * scale) : r * scale;
}

// Row i's two factors of a chain.
struct XaTerm {
    int kind;
    const float *q, *y;
    const double *v;
    bool cg;  // v was written by other blocks of this launch: read it through L2
    __device__ __forceinline__ void operator()(int i, double &a, double &b) const
    {
        if (kind == XA_QY) {
            a = xc_f2d(q[i]);
            b = xc_f2d(y[i]);
            return;
        }
        const double vi = cg ? __ldcg(v + i) : v[i];
        a = kind == XA_SQ ? vi : xc_f2d(q[i]);
        b = vi;
    }
};



// Exclusive prefix over the block (thread order) and the block total; every
// thread calls it. `sh` holds XA_NW + 1 doubles.
__device__ double block_excl(double v, double *sh, double &total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) {
            inc += u;
        }
    }
    if (lane == 31) {
        sh[warp] = inc;
    }
    __syncthreads();
    if (warp == 0) {
        double w = lane < XA_NW ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) {
                w += u;
            }
        }
        if (lane < XA_NW) {
            sh[lane] = w;
        }
    }
    __syncthreads();
    total = sh[XA_NW - 1];
    const double ex = (warp > 0 ? sh[warp - 1] : 0.0) + (inc - v);
    __syncthreads();
    return ex;
}

__global__ void __launch_bounds__(XA_T, 2) k_xappend(const XaArgs A)
{
    // records: this block's chunks, sub-groups and warps; in the last block
    // also the blocks' records (over the chunks') and one block's sub-records
    // for a descent (xa_smem_bytes)
    extern __shared__ __align__(16) unsigned char xa_smem[];
    XcRec *const s_rc = reinterpret_cast<XcRec *>(xa_smem);
    XcRec *const s_rs = s_rc + XA_T;
    XcRec *const s_rw = s_rs + XA_NS;
    XcRecB *const s_rbk = reinterpret_cast<XcRecB *>(xa_smem);
    XcRec *const d_rc = reinterpret_cast<XcRec *>(xa_smem + XA_SMEM_OWN);
    XcRec *const d_rs = d_rc + XA_T;
    XcRec *const d_rw = d_rs + XA_NS;
    __shared__ XcRecB s_rb;
    __shared__ XcRecB s_rg[XA_MAXG / XA_GRP];
    __shared__ double s_sh[XA_NW + 1];
    __shared__ double s_agg[3][XA_NW];
    __shared__ double s_t;
    __shared__ int s_last, s_ok;

    const int t = threadIdx.x, lane = t & 31, warp = t >> 5, b = blockIdx.x, G = gridDim.x;
    const int n = A.n, L = A.L, ch = blockIdx.y;
    const float *const Aq = A.q ? A.q + (size_t)(ch % A.qk) * A.qld : nullptr;
    const float *const Ay =
        A.y ? A.y + (size_t)(A.ycol ? A.ycol[ch / A.qk] : ch / A.qk) * A.yld : nullptr;
    XcRec *const Arc = A.rc + (size_t)ch * G * XA_T;
    XcRec *const Ars = A.rs + (size_t)ch * G * XA_NS;
    XcRec *const Arw = A.rw + (size_t)ch * G * XA_NW;
    XcRecB *const Arb = A.rb + (size_t)ch * G;
    double *const Aagg = A.agg + (size_t)ch * 3 * G;
    const double *const Ag_in = A.g_in + (size_t)ch * G;
    double *const Ag_out = A.g_out + (size_t)ch * G;
    unsigned *const Aticket = A.ticket + ch;
    auto rows_lo = [&](int gt) { return (int)min((long long)n, (long long)gt * L); };
    auto rows_hi = [&](int gt) { return (int)min((long long)n, (long long)gt * L + L); };
    const int gt = b * XA_T + t, i0 = rows_lo(gt), i1 = rows_hi(gt);
    const bool chain = A.kind != XA_NONE;

    // 1. row operations, the chain's chunk sum, the next chain's aggregates
    const double cprev = A.upd ? A.res[A.c_slot] : 0.0;
    const float raw = A.scale ? (float)sqrt(A.res[R_RAW2]) : 1.0f;
    const double w = A.norm ? sqrt(A.res[A.w_slot]) : 1.0;
    const float sx = A.fill ? A.s[A.xcol] : 0.0f;
    float *Bm = A.B + (size_t)A.mcol * n;
    const float *Bp = A.B + (size_t)A.bcol * n;
    const float *Xc = A.X + (size_t)A.xcol * A.ldX;
    XcGuess gs, g0, g1, g2;
    const bool need_q = chain && A.kind != XA_SQ;  // this chain's column (QV, QY)
    const bool need_y = A.kind == XA_QY || A.next == XN_QY || A.next == XN_AB;
    const bool need_qc = need_q || A.next == XN_QV_UPD || A.next == XN_SQ_UPD || A.next == XN_AB;
    // Tiles of XA_TILE rows: every load of a tile is issued before its rows are
    // used (the rows of a thread are consecutive, so a warp's loads are strided).
    for (int base = i0; base < i1; base += XA_TILE) {
        float xs[XA_TILE], bs[XA_TILE], qp[XA_TILE], qc[XA_TILE], qn[XA_TILE], ys[XA_TILE],
            bm[XA_TILE];
        double vin[XA_TILE];
#pragma unroll
        for (int u = 0; u < XA_TILE; ++u) {
            const int i = min(base + u, i1 - 1);  // past the chunk: row i1 - 1 again, unused
            if (A.fill) {
                xs[u] = Xc[i];
                bs[u] = Bp[i];
                vin[u] = 0.0;
            } else {
                vin[u] = A.v_in ? A.v_in[i] : 0.0;
                if (A.scale) {
                    bm[u] = Bm[i];
                }
            }
            if (A.upd) {
                qp[u] = A.q_prev[i];
            }
            if (need_qc) {
                qc[u] = Aq[i];
            }
            if (A.next == XN_QV || A.next == XN_QV_UPD) {
                qn[u] = A.q_next[i];
            }
            if (need_y) {
                ys[u] = Ay[i];
            }
        }
#pragma unroll
        for (int u = 0; u < XA_TILE; ++u) {
            const int i = base + u;
            if (i >= i1) {
                continue;
            }
            double v = vin[u];
            if (A.fill) {
                float val;
                if (A.type == 'l') {
                    val = sx * bs[u] * xs[u];
                } else {
                    const float d = (A.type == '+') ? xs[u] - A.h : A.h - xs[u];
                    val = sx * bs[u] * ((d < 0.0f) ? 0.0f : d);  // std::max(d, 0.0f)
                }
                Bm[i] = val;
                v = xc_f2d(val);
            } else if (A.scale) {
                Bm[i] = bm[u] / raw;
            }
            if (A.upd) {
                v = fma(-cprev, xc_f2d(qp[u]), v);
            }
            float qo = 0.0f;
            if (A.norm) {
                v = v / w;
                qo = (float)v;
                if (A.q_out) {
                    A.q_out[i] = qo;
                }
            }
            if (A.v_out) {
                A.v_out[i] = v;
            }
            float vh, vl;
            ff_of(v, vh, vl);
            if (chain) {
                if (A.kind == XA_SQ) {
                    gs.add_scaled(vh, vh, 2.0f * vl);
                } else if (A.kind == XA_QV) {
                    gs.add_scaled(qc[u], vh, vl);
                } else {
                    gs.add_product(qc[u], ys[u]);
                }
            }
            switch (A.next) {
            case XN_SQ:
                g0.add_scaled(vh, vh, 2.0f * vl);
                break;
            case XN_QV:
                g0.add_scaled(qn[u], vh, vl);
                break;
            case XN_QY:
                g0.add_product(qo, ys[u]);
                break;
            case XN_AB:
                g0.add_product(qc[u], ys[u]);
                break;
            case XN_QV_UPD:
                g0.add_scaled(qn[u], vh, vl);
                g1.add_product(-qn[u], qc[u]);
                break;
            case XN_SQ_UPD:
                g0.add_scaled(vh, vh, 2.0f * vl);
                g1.add_scaled(-2.0f * qc[u], vh, vl);
                g2.add_product(qc[u], qc[u]);
                break;
            default:
                break;
            }
        }
    }
    if (A.next != XN_NONE) {
        const double a[3] = {g0.value(), g1.value(), g2.value()};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double r = warp_sum(a[k]);
            if (lane == 0) {
                s_agg[k][warp] = r;
            }
        }
    }
    __syncthreads();
    if (A.next != XN_NONE && t < 3) {
        double r = 0.0;
        for (int q = 0; q < XA_NW; ++q) {
            r += s_agg[t][q];
        }
        Aagg[(size_t)b * 3 + t] = r;
    }

    // 2. chunk guesses and speculative runs
    const double *vsrc = A.v_out ? A.v_out : A.v_in;
    if (chain) {
        double total;
        const double ex = block_excl(gs.value(), s_sh, total);
        const double guess = Ag_in[b] + ex;
        const XaTerm tm{A.kind, Aq, Ay, vsrc, false};
        XcSpecR sp;
        sp.begin(guess, guess == 0.0);
        for (int base = i0; base < i1; base += XA_TILE) {
            double xa[XA_TILE], ya[XA_TILE];
#pragma unroll
            for (int u = 0; u < XA_TILE; ++u) {
                tm(min(base + u, i1 - 1), xa[u], ya[u]);
            }
#pragma unroll
            for (int u = 0; u < XA_TILE; ++u) {
                if (base + u < i1) {
                    sp.step(xa[u], ya[u]);
                }
            }
        }
        sp.finish(s_rc[t], i1 <= i0);
        Arc[gt] = s_rc[t];
        __syncthreads();

        // 3. composition: sub-groups, warps, the block
        const XaTerm tl{A.kind, Aq, Ay, vsrc, false};
        auto rerun_local = [&](int c, double &v, XcTrack &tr) {  // chunk c of this block
            xc_run_track(tl, rows_lo(b * XA_T + c), rows_hi(b * XA_T + c), v, tr);
        };
        auto through_sub = [&](int sg, double &v, XcTrack &tr) {
            const int c0 = sg * XA_SUB;
            v = xc_walk([&](int k) -> const XcRec & { return s_rc[c0 + k]; }, XA_SUB, v, tr,
                        [&](int k, double &u, XcTrack &tq) { rerun_local(c0 + k, u, tq); });
        };
        {
            const int sg = lane >> 3, ln = lane & 7;
            if (ln < XA_LANES) {
                const int c0 = warp * 32 + sg * XA_SUB;
                xc_compose_lane([&](int k) -> const XcRec & { return s_rc[c0 + k]; }, XA_SUB, ln,
                                [&](int k, double &u, XcTrack &tq) { rerun_local(c0 + k, u, tq); },
                                s_rs[warp * 4 + sg]);
            }
        }
        __syncwarp();
        if (lane < XA_LANES) {
            xc_compose_lane([&](int k) -> const XcRec & { return s_rs[warp * 4 + k]; }, 4, lane,
                            [&](int k, double &u, XcTrack &tq) { through_sub(warp * 4 + k, u, tq); },
                            s_rw[warp]);
        }
        __syncthreads();
        if (warp == 0 && lane < XA_LANES_B) {
            xc_compose_lane(
                [&](int k) -> const XcRec & { return s_rw[k]; }, XA_NW, lane,
                [&](int k, double &u, XcTrack &tq) {
                    u = xc_walk([&](int q) -> const XcRec & { return s_rs[k * 4 + q]; }, 4, u, tq,
                                [&](int q, double &z, XcTrack &tz) { through_sub(k * 4 + q, z, tz); });
                },
                s_rb);
        }
        __syncthreads();
        if (t < XA_NS) {
            Ars[(size_t)b * XA_NS + t] = s_rs[t];
        } else if (t < XA_NS + XA_NW) {
            Arw[(size_t)b * XA_NW + t - XA_NS] = s_rw[t - XA_NS];
        } else if (t == XA_NS + XA_NW) {
            Arb[b] = s_rb;
        }
    }

    // 4. the last block
    __threadfence();
    __syncthreads();
    if (t == 0) {
        s_last = atomicAdd(Aticket, 1u) == (unsigned)G - 1u;
    }
    __syncthreads();
    if (!s_last) {
        return;
    }
    __threadfence();
    double c = 0.0;
    if (chain) {
        const XaTerm tg{A.kind, Aq, Ay, vsrc, true};
        const int ngrp = (G + XA_GRP - 1) / XA_GRP;
        // the blocks' records into shared memory (this block's chunk records are done with)
        auto copy_recs = [&](auto *dst, const auto *src, int count) {
            static_assert(sizeof(*dst) == sizeof(*src) && sizeof(*dst) % 8 == 0, "records");
            const double *sp = reinterpret_cast<const double *>(src);
            double *dp = reinterpret_cast<double *>(dst);
            for (int k = t; k < count * (int)(sizeof(*dst) / 8); k += XA_T) {
                dp[k] = __ldcg(sp + k);
            }
        };
        copy_recs(s_rbk, Arb, G);
        __syncthreads();
        // groups of XA_GRP blocks; a lane meeting a block that cannot vouch for
        // its value gives up (the final walk descends there instead)
        {
            const int g = t >> 4, ln = t & 15;
            if (g < ngrp && ln < XA_LANES_B) {
                const int b0 = g * XA_GRP, cnt = min(XA_GRP, G - b0);
                xc_compose_lane([&](int k) -> const XcRecB & { return s_rbk[b0 + k]; }, cnt, ln,
                                [&](int, double &, XcTrack &tq) { tq.lost = true; }, s_rg[g]);
            }
        }
        if (t == 0) {
            s_t = 0.0;
        }
        __syncthreads();
        // The walk from the true start 0: thread 0 steps through the group
        // records, and through a group's block records where the group's
        // cannot vouch for its value, on its own; where a block's record cannot
        // either, the block loads that block's sub-records for it and thread 0
        // walks them, re-running rows at the bottom.
        int pos_g = 0, pos_b = -1;  // thread 0: the group, the block in it (-1: none yet)
        for (;;) {
            if (t == 0) {
                int fail = -1;
                double v = s_t;
                XcTrack tr;
                tr.init(0u);
                while (fail < 0 && pos_g < ngrp) {
                    const int b0 = pos_g * XA_GRP, cnt = min(XA_GRP, G - b0);
                    if (pos_b < 0) {
                        if (xc_track(s_rg[pos_g], v, tr)) {
                            ++pos_g;
                            continue;
                        }
                        pos_b = 0;
                    }
                    while (pos_b < cnt && xc_track(s_rbk[b0 + pos_b], v, tr)) {
                        ++pos_b;
                    }
                    if (pos_b < cnt) {
                        fail = b0 + pos_b++;
                    }
                    if (pos_b >= cnt) {
                        ++pos_g;
                        pos_b = -1;
                    }
                }
                s_t = v;
                s_ok = fail;
            }
            __syncthreads();
            const int bk = s_ok;
            if (bk < 0) {
                break;
            }
            copy_recs(d_rw, Arw + (size_t)bk * XA_NW, XA_NW);
            copy_recs(d_rs, Ars + (size_t)bk * XA_NS, XA_NS);
            copy_recs(d_rc, Arc + (size_t)bk * XA_T, XA_T);
            __syncthreads();
            if (t == 0) {
                XcTrack tr;
                tr.init(0u);
                s_t = xc_walk(
                    [&](int w) -> const XcRec & { return d_rw[w]; }, XA_NW, s_t, tr,
                    [&](int w, double &u, XcTrack &tq) {
                        u = xc_walk(
                            [&](int q) -> const XcRec & { return d_rs[w * 4 + q]; }, 4, u, tq,
                            [&](int q, double &z, XcTrack &tz) {
                                const int c0 = (w * 4 + q) * XA_SUB;
                                z = xc_walk([&](int r) -> const XcRec & { return d_rc[c0 + r]; },
                                            XA_SUB, z, tz, [&](int r, double &e, XcTrack &te) {
                                                const int gch = bk * XA_T + c0 + r;
                                                xc_run_track(tg, rows_lo(gch), rows_hi(gch), e, te);
                                            });
                            });
                    });
            }
            __syncthreads();
        }
        c = s_t;
        if (t == 0) {
            A.res[A.res_slot + ch] = c;
        }
    }
    if (A.next != XN_NONE) {
        // block entry guesses of the next chain: exclusive prefix of the blocks'
        // aggregates at this chain's value, blocks t and t + XA_T
        double carry = 0.0;
        for (int base = 0; base < G; base += XA_T) {
            const int k = base + t;
            double a = 0.0;
            if (k < G) {
                const double a0 = __ldcg(Aagg + (size_t)k * 3), a1 = __ldcg(Aagg + (size_t)k * 3 + 1),
                             a2 = __ldcg(Aagg + (size_t)k * 3 + 2);
                a = a0 + c * (a1 + c * a2);
            }
            double total;
            const double ex = block_excl(a, s_sh, total);
            if (k < G) {
                Ag_out[k] = carry + ex;
            }
            carry += total;
        }
    }
    if (t == 0) {
        *Aticket = 0u;  // for the next launch (stream order)
    }
}

constexpr size_t xa_smem_bytes() { return XA_SMEM_OWN + sizeof(XcRec) * (XA_T + XA_NS + XA_NW); }

int xa_blocks(int n)
{
    static int sms = 0;
    if (sms == 0) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0) {
            sms = v;
        } else {
            sms = 152;
        }
    }
    const long long want = ((long long)n + (long long)XA_T * XA_LMIN - 1) / ((long long)XA_T * XA_LMIN);
    return (int)std::max<long long>(1, std::min<long long>(want, std::min(XA_MAXG, 2 * sms)));
}

}  // namespace

namespace {

// One append's (or one orthonormalisation's) sequence of chain launches.
struct XaRun {
    cudaStream_t st;
    int n, m, max_terms, G, L;
    const float *BoC;
    XaBufs &bf;
    long long *launches;
    int launch = 0, cur = 0;  // launches so far; the generation of the working column
    double *vb[2], *gb[2], *res;

    XaRun(cudaStream_t st_, int n_, int m_, int max_terms_, const float *BoC_, XaBufs &bf_,
          long long *launches_)
        : st(st_), n(n_), m(m_), max_terms(max_terms_), BoC(BoC_), bf(bf_), launches(launches_)
    {
        G = xa_blocks(n);
        L = (int)ceil_div((size_t)n, (size_t)G * XA_T);
        bf.v0.ensure(sizeof(double) * n);
        bf.v1.ensure(sizeof(double) * n);
        bf.rc.ensure(sizeof(XcRec) * (size_t)G * XA_T);
        bf.rs.ensure(sizeof(XcRec) * (size_t)G * XA_NS);
        bf.rw.ensure(sizeof(XcRec) * (size_t)G * XA_NW);
        bf.rb.ensure(sizeof(XcRecB) * (size_t)G);
        bf.agg.ensure(sizeof(double) * 3 * (size_t)G);
        bf.g0.ensure(sizeof(double) * (size_t)G);
        bf.g1.ensure(sizeof(double) * (size_t)G);
        bf.res.ensure(sizeof(double) * (size_t)(R_C + 2 * max_terms));
        if (bf.ticket.bytes == 0) {
            bf.ticket.ensure(sizeof(unsigned));
            CUDA_CHECK(cudaMemsetAsync(bf.ticket.ptr, 0, sizeof(unsigned), st));
        }
        vb[0] = bf.v0.as<double>();
        vb[1] = bf.v1.as<double>();
        gb[0] = bf.g0.as<double>();
        gb[1] = bf.g1.as<double>();
        res = bf.res.as<double>();
    }
    const float *col(int j) const { return BoC + (size_t)j * n; }
    XaArgs base() const
    {
        XaArgs a{};
        a.n = n;
        a.L = L;
        a.qk = 1;
        a.mcol = m;
        a.res = res;
        a.rc = bf.rc.as<XcRec>();
        a.rs = bf.rs.as<XcRec>();
        a.rw = bf.rw.as<XcRec>();
        a.rb = bf.rb.as<XcRecB>();
        a.agg = bf.agg.as<double>();
        a.ticket = bf.ticket.as<unsigned>();
        return a;
    }
    void go(XaArgs &a)
    {
        a.g_in = gb[launch & 1];
        a.g_out = gb[(launch + 1) & 1];
        allow_smem(k_xappend, xa_smem_bytes());
        k_xappend<<<(unsigned)G, XA_T, xa_smem_bytes(), st>>>(a);
        LAUNCH_CHECK();
        ++launch;
        ++*launches;
    }
    // A launch with no chain that only leaves the guesses of the first chain
    // of a pass over the column in vb[cur].
    void prime()
    {
        XaArgs a = base();
        a.v_in = vb[cur];
        if (m > 0) {
            a.next = XN_QV;
            a.q_next = col(0);
        } else {
            a.next = XN_SQ;
        }
        go(a);
    }
    // One modified Gram-Schmidt pass (kernels.cc:194-211) over the column in
    // vb[cur], whose first chain's guesses the previous launch left: chain j's
    // value to res[slot + j], then the squared norm (kernels.cc:251-255) to
    // res[vn_slot]. scale_B: the first launch also divides B[:, m] by the raw
    // norm in res[R_RAW2] (marsalgo.cc:836).
    void pass(int slot, int vn_slot, float *scale_B)
    {
        for (int j = 0; j <= m; ++j) {
            XaArgs a = base();
            if (j == 0 && scale_B) {
                a.scale = 1;
                a.B = scale_B;
            }
            if (j > 0) {
                a.upd = 1;
                a.q_prev = col(j - 1);
                a.c_slot = slot + j - 1;
                a.v_in = vb[cur];
                a.v_out = vb[cur ^ 1];
                cur ^= 1;
            } else {
                a.v_in = vb[cur];
            }
            if (j < m) {
                a.kind = XA_QV;
                a.q = col(j);
                a.res_slot = slot + j;
                if (j + 1 < m) {
                    a.next = XN_QV_UPD;
                    a.q_next = col(j + 1);
                } else {
                    a.next = XN_SQ_UPD;
                }
            } else {
                a.kind = XA_SQ;
                a.res_slot = vn_slot;
                if (m > 0) {
                    a.next = XN_QV;  // the first chain of a re-pass
                    a.q_next = col(0);
                }
            }
            go(a);
        }
    }
    // kernels.cc:239-266: a pass, and the DGKS re-pass when the projection
    // removed most of the column (the gate ratio squared, kernels.h:17).
    // Returns the squared norm of the final column; *w_slot is its slot.
    double orthonormalize(double tol, float *scale_B, bool *dgks, int *w_slot)
    {
        pass(R_C, R_VN, scale_B);
        std::vector<double> h((size_t)R_C + m);
        CUDA_CHECK(cudaMemcpyAsync(h.data(), res, sizeof(double) * h.size(),
                                   cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        double proj = 0.0;
        for (int j = 0; j < m; ++j) {
            proj = std::fma(h[R_C + j], h[R_C + j], proj);
        }
        double vn = h[R_VN];
        *w_slot = R_VN;
        *dgks = false;
        if (vn > tol && vn * 9.0 < proj) {
            *dgks = true;
            pass(R_C + max_terms, R_VN2, nullptr);
            CUDA_CHECK(cudaMemcpyAsync(&vn, res + R_VN2, sizeof(double), cudaMemcpyDeviceToHost, st));
            CUDA_CHECK(cudaStreamSynchronize(st));
            *w_slot = R_VN2;
        }
        return vn;
    }
    // v / w (kernels.cc:274-279): into q_out as f32 (and the y dot's guesses),
    // or into the other generation of the working column.
    void normalise(int w_slot, float *q_out, const float *y)
    {
        XaArgs a = base();
        a.norm = 1;
        a.w_slot = w_slot;
        a.v_in = vb[cur];
        if (q_out) {
            a.q_out = q_out;
            a.next = XN_QY;
            a.y = y;
        } else {
            a.v_out = vb[cur ^ 1];
            cur ^= 1;
        }
        go(a);
    }
};

}  // namespace

XaOutcome append_exact(cudaStream_t st, const XaFit &f, char type, int xcol, int bcol, float h,
                       XaBufs &bf, long long *launches)
{
    XaRun run(st, f.n, f.m, f.max_terms, f.BoC, bf, launches);
    const int m = f.m;
    // the column and its raw norm (marsalgo.cc:819-836)
    {
        XaArgs a = run.base();
        a.fill = 1;
        a.type = type;
        a.X = f.X;
        a.ldX = f.ldX;
        a.s = f.s;
        a.xcol = xcol;
        a.bcol = bcol;
        a.h = h;
        a.B = f.B;
        a.v_out = run.vb[0];
        a.next = XN_SQ;
        run.go(a);
    }
    {
        XaArgs a = run.base();
        a.v_in = run.vb[0];
        a.kind = XA_SQ;
        a.res_slot = R_RAW2;
        a.next = XN_QV;
        a.q_next = run.col(0);
        run.go(a);
    }
    XaOutcome out{};
    int w_slot = R_VN;
    const double vn = run.orthonormalize(f.tol, f.B, &out.dgks, &w_slot);
    out.w2 = vn;
    const double wn = std::sqrt(vn);
    if (!(wn * wn > f.tol)) {
        return out;
    }
    // column m of BoC and y . it (marsalgo.cc:846-857)
    float *q = f.BoC + (size_t)m * f.n;
    run.normalise(w_slot, q, f.y);
    {
        XaArgs a = run.base();
        a.kind = XA_QY;
        a.q = q;
        a.y = f.y;
        a.res_slot = R_YBO;
        run.go(a);
    }
    CUDA_CHECK(cudaMemcpyAsync(&out.ybo, run.res + R_YBO, sizeof(double), cudaMemcpyDeviceToHost,
                               st));
    CUDA_CHECK(cudaStreamSynchronize(st));
    out.stored = true;
    return out;
}

double orthonormalize_col_exact(cudaStream_t st, int n, int m, const float *BoC, double *v,
                                double tol, XaBufs &bf, long long *launches, bool *dgks)
{
    XaRun run(st, n, m, m + 1, BoC, bf, launches);
    CUDA_CHECK(cudaMemcpyAsync(run.vb[0], v, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    run.prime();
    int w_slot = R_VN;
    const double vn = run.orthonormalize(tol, nullptr, dgks, &w_slot);
    const double w = std::sqrt(vn);
    if (w * w > tol) {
        run.normalise(w_slot, nullptr, nullptr);
    }
    CUDA_CHECK(cudaMemcpyAsync(v, run.vb[run.cur], sizeof(double) * n, cudaMemcpyDeviceToDevice,
                               st));
    return w;
}

// T = Bo^T Bx for few candidates (kernels.cc:327-335): the chain of entry
// q = j m + k is sum_i BoC[i, k] Bx[i, col(j)], rows in order, for all of them
// side by side (blockIdx.y), each evaluated exactly in parallel. Two launches:
// the blocks' sums of the terms (entry guesses), then the chains.
bool tgemm_exact(cudaStream_t st, int n, int m, int P, const float *BoC, const float *Bx,
                 size_t ldBx, const int *col, double *T, XaBufs &bf, long long *launches)
{
    const long long chains = (long long)P * m;
    if (n <= 0 || chains <= 0 || chains > XA_MAX_CHAINS) {
        return false;
    }
    // blocks per chain: at least 16 rows a chunk; records of all chains
    // within XA_REC_BUDGET bytes
    const size_t per_block = sizeof(XcRec) * (XA_T + XA_NS + XA_NW) + sizeof(XcRecB);
    const long long gmax =
        std::max<long long>(1, (long long)(XA_REC_BUDGET / ((size_t)chains * per_block)));
    const int G = (int)std::max<long long>(1, std::min<long long>(xa_blocks(n), gmax));
    const int L = (int)ceil_div((size_t)n, (size_t)G * XA_T);
    const size_t cg = (size_t)chains * G;
    bf.rc.ensure(sizeof(XcRec) * cg * XA_T);
    bf.rs.ensure(sizeof(XcRec) * cg * XA_NS);
    bf.rw.ensure(sizeof(XcRec) * cg * XA_NW);
    bf.rb.ensure(sizeof(XcRecB) * cg);
    bf.agg.ensure(sizeof(double) * 3 * cg);
    bf.g0.ensure(sizeof(double) * cg);
    bf.g1.ensure(sizeof(double) * cg);
    if (bf.ticket.bytes < sizeof(unsigned) * (size_t)chains) {
        bf.ticket.ensure(sizeof(unsigned) * (size_t)chains);
        CUDA_CHECK(cudaMemsetAsync(bf.ticket.ptr, 0, bf.ticket.bytes, st));
    }
    XaArgs a{};
    a.n = n;
    a.L = L;
    a.q = BoC;
    a.qk = m;
    a.qld = (size_t)n;
    a.y = Bx;
    a.yld = ldBx;
    a.ycol = col;
    a.res = T;
    a.rc = bf.rc.as<XcRec>();
    a.rs = bf.rs.as<XcRec>();
    a.rw = bf.rw.as<XcRec>();
    a.rb = bf.rb.as<XcRecB>();
    a.agg = bf.agg.as<double>();
    a.ticket = bf.ticket.as<unsigned>();
    const dim3 grid((unsigned)G, (unsigned)chains);
    allow_smem(k_xappend, xa_smem_bytes());
    a.next = XN_AB;  // the guesses
    a.g_out = bf.g0.as<double>();
    k_xappend<<<grid, XA_T, xa_smem_bytes(), st>>>(a);
    LAUNCH_CHECK();
    a.next = XN_NONE;  // the chains
    a.kind = XA_QY;
    a.res_slot = 0;
    a.g_in = bf.g0.as<double>();
    a.g_out = bf.g1.as<double>();
    k_xappend<<<grid, XA_T, xa_smem_bytes(), st>>>(a);
    LAUNCH_CHECK();
    *launches += 2;
    return true;
}

}  // namespace mgpu
