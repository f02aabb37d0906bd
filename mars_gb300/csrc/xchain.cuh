// Exact parallel evaluation of a sequential FP64 accumulation
//
//     acc_0 = 0,   acc_{i+1} = fma((double)a_i, (double)b_i, acc_i),   i = 0 .. n-1,
//
// with a_i, b_i f32: the order the reference uses for its column norms and dot
// products (kernels.cc:215-237 dot_widen, kernels.cc:361-366 the norm of the
// stored column, marsalgo.cc:359-369 the column norms of X). Run as written, the
// chain costs n times the FP64 FMA latency (~67 cycles on GB300: 32 ms for 10^6
// rows), whatever the number of chains.
//
// Why a parallel form exists. Let acc lie on the grid of multiples of u, and let
// the exact sum acc + a b lie in a binade whose ulp is u. Then fma(a, b, acc) =
// acc + u r, where r is a b / u rounded to the nearest integer and a tie goes to
// whichever neighbour makes acc / u + r even. The step is a translation whose
// offset depends on the parity of acc / u only. So if a run of steps from a start
// s passes through binades whose largest ulp is U, then from s + d, with d a
// multiple of 2 U, every step rounds on the same grid with the same ties, and the
// run ends at (the run's end from s) + d, provided each exact sum of the shifted
// run stays in the binade of the unshifted one.
//
// The rows are cut into chunks:
//  1. the chunk's terms are summed in float-float (FP32 pipe); a prefix of those
//     sums guesses the value the accumulation has when it enters each chunk;
//  2. each chunk runs the true recurrence XC_RUNS = 4 times, from the guess with
//     its two last mantissa bits set to 0, 1, 2, 3 (the residues modulo 4 ulps of
//     the start's binade), and records each run's end and how far its values kept
//     from the edges of their binades (xc_speculate). Four residues let a run
//     climb one binade above its start; it may fall any number;
//  3. the chunks are walked in order with the true value t (xc_resolve): where t
//     is in the binade of the chunk's start, the run with t's residue applies if
//     |t - its start| is inside that run's margin, and the chunk's end is the
//     run's end plus (t - its start), an exact FP64 add; where t is +0 (a chain
//     whose terms have all been zero so far, as a hinge parent's are on one side
//     of its knot), a fifth run from +0 gives the end directly; anywhere else the
//     chunk is re-run from t in order.
// The result equals the sequential recurrence bit for bit whatever the data (NaN,
// infinities, zeros, subnormals, sign changes included): every chunk the checks
// cannot vouch for is recomputed in order.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define XC_HD __host__ __device__ __forceinline__
#define XC_UNROLL _Pragma("unroll")
#define XC_UNROLL4 _Pragma("unroll 4")
#else
#include <cmath>
#include <cstring>
#define XC_HD inline
#define XC_UNROLL
#define XC_UNROLL4
#endif

XC_HD uint32_t xc_hi(double v)
{
#ifdef __CUDA_ARCH__
    return (uint32_t)__double2hiint(v);
#else
    uint64_t b;
    memcpy(&b, &v, 8);
    return (uint32_t)(b >> 32);
#endif
}

XC_HD uint32_t xc_lo(double v)
{
#ifdef __CUDA_ARCH__
    return (uint32_t)__double2loint(v);
#else
    uint64_t b;
    memcpy(&b, &v, 8);
    return (uint32_t)b;
#endif
}

XC_HD double xc_words(uint32_t hi, uint32_t lo)
{
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)hi, (int)lo);
#else
    const uint64_t b = ((uint64_t)hi << 32) | lo;
    double v;
    memcpy(&v, &b, 8);
    return v;
#endif
}

// The f64 value of an f32, exactly. On the device it is built from the bit
// fields on the integer pipe: GB300 issues conversions to f64 on its narrow
// FP64 pipe, which the chains' fused multiply-adds keep busy. Subnormal floats
// take the conversion.
XC_HD double xc_f2d(float f)
{
#ifdef __CUDA_ARCH__
    const uint32_t b = __float_as_uint(f), e = (b >> 23) & 0xffu, mant = b & 0x7fffffu;
    if (e == 0u && mant != 0u) {
        return (double)f;
    }
    const uint32_t de = e == 0u ? 0u : (e == 0xffu ? 0x7ffu : e + 896u);
    return __hiloint2double((int)((b & 0x80000000u) | (de << 20) | (mant >> 3)), (int)(mant << 29));
#else
    return (double)f;
#endif
}

XC_HD uint32_t xc_umin(uint32_t a, uint32_t b) { return a < b ? a : b; }
XC_HD uint32_t xc_umax(uint32_t a, uint32_t b) { return a > b ? a : b; }

constexpr int XC_RUNS = 4;

// What one chunk's speculative runs leave for the walk.
struct XcChunk {
    double start;            // the guess with its two last mantissa bits cleared
    double end[XC_RUNS];     // end of the run from start + r ulps
    double margin[XC_RUNS];  // largest |t - (start + r ulps)| run r vouches for, or -1
    double zero_end;         // end of the run from +0 (a chain still at its start value)
};

// Margin of one run. h0 is the high word of its start; [hmin, hmax] the range of
// the magnitude high words (sign bit cleared) of the values it produced; edge is
// set when one of those values had the 20 mantissa bits of its high word all zero
// or all one, i.e. lay within 2^(e-20) of an edge of its binade [2^e, 2^(e+1)) in
// magnitude. Otherwise every value keeps 2^(e_lo - 20) from the edges of its own
// binade (e_lo the lowest binade visited), zero included, and a shift by d keeps
// each exact sum in the binade of the unshifted one -- same sign, same exponent --
// when |d| <= 2^(e_lo - 20) - 2 U, U = 2^(e_hi - 52) the largest ulp visited. The
// values may change sign: no shifted sum crosses zero, since every one keeps
// farther than |d| from it. The run may end at most one binade above its start
// (U <= 2 ulps of the start), so that the residue modulo 4 ulps makes d a
// multiple of 2 U. An empty run vouches for any d.
XC_HD double xc_margin(uint32_t h0, uint32_t hmin, uint32_t hmax, bool edge, bool empty)
{
    if (empty) {
        return 1.0e300;
    }
    const uint32_t E0 = (h0 >> 20) & 0x7ffu, Elo = (hmin >> 20) & 0x7ffu,
                   Ehi = (hmax >> 20) & 0x7ffu;
    if (edge || E0 < 64u || Elo < 64u || Ehi > 2045u || Ehi > E0 + 1u || Ehi < Elo) {
        return -1.0;
    }
    const double m = xc_words((Elo - 20u) << 20, 0u) - xc_words((Ehi - 51u) << 20, 0u);
    return m >= 0.0 ? m : -1.0;
}

// The XC_RUNS speculative runs of one chain through one chunk: begin() from the
// guess, step() once per row with the row's two FP64 factors (exact products of
// f32 values, or a lower-level chain's value times an exact factor), finish()
// into the chunk's record.
struct XcSpec {
    double a[XC_RUNS], z;
    uint32_t mn[XC_RUNS], mx[XC_RUNS], ed[XC_RUNS];
    uint32_t h0, l0;
    XC_HD void begin(double guess)
    {
        z = 0.0;
        h0 = xc_hi(guess);
        l0 = xc_lo(guess) & ~(uint32_t)(XC_RUNS - 1);
XC_UNROLL
        for (int r = 0; r < XC_RUNS; ++r) {
            a[r] = xc_words(h0, l0 | (uint32_t)r);
            mn[r] = 0xffffffffu;
            mx[r] = 0u;
            ed[r] = 0u;
        }
    }
    XC_HD void step(double x, double y)
    {
        z = fma(x, y, z);
XC_UNROLL
        for (int r = 0; r < XC_RUNS; ++r) {
            a[r] = fma(x, y, a[r]);
            const uint32_t h = xc_hi(a[r]) & 0x7fffffffu;
            mn[r] = xc_umin(mn[r], h);
            mx[r] = xc_umax(mx[r], h);
            ed[r] |= (uint32_t)(((h + 1u) & 0xfffffu) < 2u);
        }
    }
    XC_HD void finish(XcChunk &c, bool empty) const
    {
        c.zero_end = z;
        c.start = xc_words(h0, l0);
XC_UNROLL
        for (int r = 0; r < XC_RUNS; ++r) {
            c.end[r] = a[r];
            c.margin[r] = xc_margin(h0, mn[r], mx[r], ed[r] != 0u, empty);
        }
    }
};

// The speculative runs of rows [i0, i1) from `guess`. term(i, a, b) yields the
// f32 factors of row i.
template <class Term>
XC_HD void xc_speculate(const Term &term, int i0, int i1, double guess, XcChunk &c)
{
    XcSpec sp;
    sp.begin(guess);
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        float x, y;
        term(i, x, y);
        sp.step(xc_f2d(x), xc_f2d(y));
    }
    sp.finish(c, i1 <= i0);
}

// The rows [i0, i1) in order from t: the reference's recurrence as written.
template <class Term>
XC_HD double xc_run(const Term &term, int i0, int i1, double t)
{
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        float x, y;
        term(i, x, y);
        t = fma(xc_f2d(x), xc_f2d(y), t);
    }
    return t;
}

// The value after a chunk given the true value t before it, from the chunk's
// record; rerun(t) runs the chunk in order where the record cannot vouch for
// the translation, and *redone is then set.
template <class Rerun>
XC_HD double xc_resolve_with(const XcChunk &c, double t, const Rerun &rerun, bool *redone)
{
    if (xc_hi(t) == 0u && xc_lo(t) == 0u) {
        return c.zero_end;  // t is +0: the run from +0 is the chain itself
    }
    const uint32_t hs = xc_hi(c.start);
    if ((xc_hi(t) >> 20) == (hs >> 20)) {
        const uint32_t r = xc_lo(t) & (uint32_t)(XC_RUNS - 1);
        const double d = t - xc_words(hs, xc_lo(c.start) | r);  // exact: one binade
        if (fabs(d) <= c.margin[r]) {
            return c.end[r] + d;  // exact: the shifted end is representable
        }
    }
    *redone = true;
    return rerun(t);
}

template <class Term>
XC_HD double xc_resolve(const Term &term, int i0, int i1, const XcChunk &c, double t,
                        bool *redone)
{
    return xc_resolve_with(c, t, [&](double v) { return xc_run(term, i0, i1, v); }, redone);
}

// Float-float accumulation of exact f32 products, for the guesses.
struct XcGuess {
    float hi = 0.f, lo = 0.f;
    XC_HD void add_product(float x, float y)
    {
#ifdef __CUDA_ARCH__
        const float ph = __fmul_rn(x, y);  // kept apart from the add below
#else
        const float ph = x * y;
#endif
        const float pl = fmaf(x, y, -ph);
        const float s = hi + ph;
        const float bb = s - hi;
        const float e = (hi - (s - bb)) + (ph - bb);
        const float t = e + (lo + pl);
        hi = s + t;
        lo = t - (hi - s);
    }
    // the sum += d * v, d f32, v a float-float value
    XC_HD void add_scaled(float d, float vh, float vl)
    {
#ifdef __CUDA_ARCH__
        const float ph = __fmul_rn(d, vh);
#else
        const float ph = d * vh;
#endif
        const float pl = fmaf(d, vh, -ph) + d * vl;
        const float s = hi + ph;
        const float bb = s - hi;
        const float e = (hi - (s - bb)) + (ph - bb);
        const float t = e + (lo + pl);
        hi = s + t;
        lo = t - (hi - s);
    }
    XC_HD void set(double v)
    {
        hi = (float)v;
        lo = (float)(v - (double)hi);
    }
    XC_HD double value() const { return (double)hi + (double)lo; }
};

// ---------------------------------------------------------------------------
// Records of a range of rows, composed level by level
//
// A record states what the chain does over its rows. For an entry t in the
// binade of `start` (same sign and exponent) whose last two mantissa bits are r,
// with |t - (start + r ulps)| <= margin[r], the chain leaves the rows at
// end[r] + (t - (start + r ulps)), exactly; from the entry +0 it leaves at
// zero_end when zero_ok. An empty record (no rows) leaves every entry as it is.
//
// A chunk's record comes from its speculative runs (XcSpecR). Consecutive
// records compose into one (xc_compose_lane): walk them from start + r ulps,
// translating through each. The composite vouches for a shift D of its entry
// (a multiple of 4 ulps of its start) when every record it walked vouches for
// the walk's own offset there plus D -- then every value of the shifted chain
// keeps the binade of the walked one -- and when no value of the walk lies more
// than one binade above the composite's start, so that D is a multiple of twice
// every ulp the shifted chain rounds to and every rounding, ties included, is
// translated. hmax[r] carries that largest magnitude up the levels.
// ---------------------------------------------------------------------------
//
// A record may carry R residues (R a power of two, its start's log2 R last
// bits clear): a composite with R residues vouches for shifts that are
// multiples of R ulps of its start, so its values may rise log2(R) - 1
// binades above it.
template <int R>
struct XcRecT {
    double start;
    double end[R];
    double margin[R];
    double zero_end;
    uint32_t hmax[R];  // largest magnitude high word visited from start + r ulps
    int zero_ok;
    int empty;
};
using XcRec = XcRecT<XC_RUNS>;

template <int R>
struct XcLog2 {
    static constexpr int value = 1 + XcLog2<R / 2>::value;
};
template <>
struct XcLog2<1> {
    static constexpr int value = 0;
};

// The XC_RUNS residue runs of one chunk, and the run from +0 when asked for
// (a chunk whose guessed entry is exactly 0).
struct XcSpecR {
    double a[XC_RUNS], z;
    uint32_t mn[XC_RUNS], mx[XC_RUNS], ed[XC_RUNS];
    uint32_t h0, l0;
    bool zero;
    XC_HD void begin(double guess, bool with_zero)
    {
        zero = with_zero;
        z = 0.0;
        h0 = xc_hi(guess);
        l0 = xc_lo(guess) & ~(uint32_t)(XC_RUNS - 1);
XC_UNROLL
        for (int r = 0; r < XC_RUNS; ++r) {
            a[r] = xc_words(h0, l0 | (uint32_t)r);
            mn[r] = 0xffffffffu;
            mx[r] = 0u;
            ed[r] = 0u;
        }
    }
    XC_HD void step(double x, double y)
    {
        if (zero) {
            z = fma(x, y, z);
        }
XC_UNROLL
        for (int r = 0; r < XC_RUNS; ++r) {
            a[r] = fma(x, y, a[r]);
            const uint32_t h = xc_hi(a[r]) & 0x7fffffffu;
            mn[r] = xc_umin(mn[r], h);
            mx[r] = xc_umax(mx[r], h);
            ed[r] |= (uint32_t)(((h + 1u) & 0xfffffu) < 2u);
        }
    }
    XC_HD void finish(XcRec &c, bool empty) const
    {
        c.start = xc_words(h0, l0);
        c.zero_end = z;
        c.zero_ok = (zero || empty) ? 1 : 0;
        c.empty = empty ? 1 : 0;
XC_UNROLL
        for (int r = 0; r < XC_RUNS; ++r) {
            c.end[r] = a[r];
            c.margin[r] = xc_margin(h0, mn[r], mx[r], ed[r] != 0u, empty);
            c.hmax[r] = xc_umax(h0 & 0x7fffffffu, mx[r]);
        }
    }
};

XC_HD bool xc_is_pzero(double t) { return xc_hi(t) == 0u && xc_lo(t) == 0u; }

// What a shift D of a walk's entry may be: every value of the walk keeps its
// binade under it while |D| <= M, and H is the largest magnitude high word the
// walk visited; ok is cleared where some value lies too near an edge of its
// binade (or zero) to allow any shift. A through() that cannot carry the walk
// (its records out of reach) sets lost instead.
struct XcTrack {
    double M;
    uint32_t H;
    bool ok;
    bool lost;  // a through() gave up: the walk's value is not the chain's
    XC_HD void init(uint32_t h)
    {
        M = 1.0e300;
        H = h & 0x7fffffffu;
        ok = true;
        lost = false;
    }
};

// Extends a walk at t through record c, if c vouches for t.
template <int R>
XC_HD bool xc_track(const XcRecT<R> &c, double &t, XcTrack &tr)
{
    if (c.empty) {
        return true;
    }
    if (xc_is_pzero(t)) {
        if (!c.zero_ok) {
            return false;
        }
        t = c.zero_end;  // a walk from another entry that reached +0 has lost its margin already
        return true;
    }
    const uint32_t hc = xc_hi(c.start);
    if ((xc_hi(t) >> 20) != (hc >> 20)) {
        return false;
    }
    const uint32_t r = xc_lo(t) & (uint32_t)(R - 1);
    const double d = t - xc_words(hc, xc_lo(c.start) | r);  // exact: one binade
    const double md = c.margin[r];
    if (!(fabs(d) <= md)) {
        return false;
    }
    tr.M = fmin(tr.M, md - fabs(d));  // exact: multiples of the start's ulp, < 2^33 of them
    tr.H = xc_umax(tr.H, c.hmax[r]);
    t = c.end[r] + d;  // exact: the shifted end keeps its binade
    return true;
}

// Extends a walk at t through rows [i0, i1) run in order; term(i, x, y) yields
// row i's two FP64 factors. The values are tracked like a run's: a shift by D
// keeps every exact sum in its binade when |D| <= 2^(e_lo - 20) - 2 U.
template <class Term>
XC_HD void xc_run_track(const Term &term, int i0, int i1, double &t, XcTrack &tr)
{
    if (i1 <= i0) {
        return;
    }
    uint32_t mn = 0xffffffffu, mx = 0u, ed = 0u;
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        double x, y;
        term(i, x, y);
        t = fma(x, y, t);
        const uint32_t h = xc_hi(t) & 0x7fffffffu;
        mn = xc_umin(mn, h);
        mx = xc_umax(mx, h);
        ed |= (uint32_t)(((h + 1u) & 0xfffffu) < 2u);
    }
    const uint32_t Elo = (mn >> 20) & 0x7ffu, Ehi = (mx >> 20) & 0x7ffu;
    if (ed || Elo < 64u || Ehi > 2045u || Ehi < Elo) {
        tr.ok = false;
    } else {
        const double m = xc_words((Elo - 20u) << 20, 0u) - xc_words((Ehi - 51u) << 20, 0u);
        if (m >= 0.0) {
            tr.M = fmin(tr.M, m);
        } else {
            tr.ok = false;
        }
    }
    tr.H = xc_umax(tr.H, mx);
}

// The walk at t through the consecutive records rec(0 .. K-1); where a record
// cannot vouch for the walk's value, through(k, t, tr) carries the walk across
// that record's rows another way (its sub-records, or the rows in order) and
// tracks it. The walk ends at the true chain value unless a through() gave up.
template <class RecAt, class Through>
XC_HD double xc_walk(const RecAt &rec, int K, double t, XcTrack &tr, const Through &through)
{
    for (int k = 0; k < K; ++k) {
        if (!xc_track(rec(k), t, tr)) {
            through(k, t, tr);
        }
    }
    return t;
}

// One lane of the composition of the consecutive records rec(0 .. K-1) into a
// record with R residues: lane r < R walks from start + r ulps and fills
// end[r], margin[r], hmax[r]; lane R walks from +0 (when the start is +0) and
// fills zero_end and
// zero_ok; lane 0 also sets
// start and empty. The lanes write disjoint fields of `out`. A walked value is
// the true chain from its entry (through() re-runs what no record vouches for,
// or gives up, and the lane's result is then marked invalid); the composite
// vouches for a shift D of the entry when every value kept its binade under it
// and no value lay more than log2(R) - 1 binades above the start.
template <class RecAt, class Through, int R>
XC_HD void xc_compose_lane(const RecAt &rec, int K, int lane, const Through &through,
                           XcRecT<R> &out)
{
    int k0 = 0;
    while (k0 < K && rec(k0).empty) {
        ++k0;
    }
    if (k0 == K) {  // no rows at all
        if (lane == 0) {
            out.start = 0.0;
            out.empty = 1;
        }
        if (lane < R) {
            out.end[lane] = 0.0;
            out.margin[lane] = 1.0e300;
            out.hmax[lane] = 0u;
        } else {
            out.zero_end = 0.0;
            out.zero_ok = 1;
        }
        return;
    }
    const double S0 = rec(k0).start;  // its last log2 R bits cleared: the composite's start
    const double S = xc_words(xc_hi(S0), xc_lo(S0) & ~(uint32_t)(R - 1));
    const uint32_t hs = xc_hi(S);
    if (lane == 0) {
        out.start = S;
        out.empty = 0;
    }
    const uint32_t Es = (hs >> 20) & 0x7ffu;
    XcTrack tr;
    tr.init(hs);
    if (lane >= R) {
        // Only a composite guessed to start at exactly 0 (every term before it
        // summed to 0) is likely to be entered at +0; other ones are descended
        // into when that happens.
        const bool z = xc_is_pzero(S);
        out.zero_end = z ? xc_walk(rec, K, 0.0, tr, through) : 0.0;
        out.zero_ok = (z && !tr.lost) ? 1 : 0;
        return;
    }
    if (Es < 64u) {  // a start this small vouches for no shift
        out.end[lane] = S;
        out.hmax[lane] = hs & 0x7fffffffu;
        out.margin[lane] = -1.0;
        return;
    }
    const double t = xc_walk(rec, K, xc_words(hs, xc_lo(S) | (uint32_t)lane), tr, through);
    const uint32_t Eh = (tr.H >> 20) & 0x7ffu;
    out.end[lane] = t;
    out.hmax[lane] = tr.H;
    out.margin[lane] =
        (tr.ok && !tr.lost && Eh <= Es + (uint32_t)(XcLog2<R>::value - 1)) ? tr.M : -1.0;
}
