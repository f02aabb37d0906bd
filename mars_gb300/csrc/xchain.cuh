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
// the high words of the values it produced (unsigned order: the order of
// magnitudes for one sign); edge is set when one of those values had the 20
// mantissa bits of its high word all zero or all one, i.e. lay within 2^(e-20) of
// an edge of its binade [2^e, 2^(e+1)). Otherwise every value keeps 2^(e_lo - 20)
// from the edges of its own binade (e_lo the lowest binade visited), and a shift
// by d keeps each exact sum in the binade of the unshifted one when
// |d| <= 2^(e_lo - 20) - 2 U, U = 2^(e_hi - 52) the largest ulp visited. The run
// may end at most one binade above its start (U <= 2 ulps of the start), so that
// the residue modulo 4 ulps makes d a multiple of 2 U. An empty run vouches for
// any d.
XC_HD double xc_margin(uint32_t h0, uint32_t hmin, uint32_t hmax, bool edge, bool empty)
{
    if (empty) {
        return 1.0e300;
    }
    const uint32_t E0 = (h0 >> 20) & 0x7ffu, Elo = (hmin >> 20) & 0x7ffu,
                   Ehi = (hmax >> 20) & 0x7ffu;
    if (edge || ((hmin ^ h0) >> 31) != 0u || ((hmax ^ h0) >> 31) != 0u || E0 < 64u ||
        Elo < 64u || Ehi > 2045u || Ehi > E0 + 1u) {
        return -1.0;
    }
    return xc_words((Elo - 20u) << 20, 0u) - xc_words((Ehi - 51u) << 20, 0u);
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
            const uint32_t h = xc_hi(a[r]);
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
        sp.step((double)x, (double)y);
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
        t = fma((double)x, (double)y, t);
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
