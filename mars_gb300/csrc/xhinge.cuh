// The hinge sweep's scalar recurrences (marsalgo.cc:91-151 covariates_impl, used
// at marsalgo.cc:603-626), chunked over the rows with the exact speculation of
// xchain.cuh. Per row i of the descending sort, with the previous row's values
// on the right-hand sides,
//     k0 += d^2 b2;  k1 += 2d bd;  w += d vb;  bd += d b2;  b2 += bk^2;  vb += yk bk
// (d = x[i-1] - x[i] in f32, rows i >= 1; row 0 sets b2 = bk^2, vb = bk yk, which
// is fma from 0 since those products are exact). The chains form three levels:
// b2, vb (terms: exact products of f32 values); bd, w, k0 (terms: an exact factor
// times b2 or vb of the previous row); k1 (2d times bd). Level by level, each
// chunk guesses its entry values in float-float from the exact entry values of
// the levels below, runs XC_RUNS speculative runs per chain with the lower levels
// re-run exactly beside them, and the chunks are walked in order. A last pass
// re-runs every chain from its chunk's exact entry values and emits k0, k1, w at
// the grid rows. Each value equals the sequential recurrence bit for bit.
//
// The routines below take one chunk [i0, i1); the kernel and the host tests call
// the same code.
#pragma once
#include "xchain.cuh"

#ifdef __CUDA_ARCH__
#define XH_LD(p) __ldg(p)
#else
#define XH_LD(p) (*(p))
#endif

// The rows of one candidate: its parent column, y and the input column, all in
// the input column's descending order.
struct XhRows {
    const float *b, *y, *x;
    XC_HD float bk(int i) const { return XH_LD(b + i); }
    XC_HD float yk(int i) const { return XH_LD(y + i); }
    XC_HD float dl(int i) const { return XH_LD(x + i - 1) - XH_LD(x + i); }  // i >= 1
};

enum { XH_B2 = 1, XH_VB = 2, XH_BD = 4, XH_W = 8, XH_K0 = 16, XH_K1 = 32, XH_ALL = 63 };
enum { XS_B2 = 0, XS_VB, XS_BD, XS_W, XS_K0, XS_K1, XS_N };

struct XhState {
    double v[XS_N];
};

// The chains selected by M through rows [i0, i1), in order, as the reference
// runs them. A chain in M needs the chains its terms read (bd, k0: b2; w: vb;
// k1: bd and b2).
template <int M>
XC_HD void xh_run(const XhRows &R, int i0, int i1, XhState &s)
{
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        const double bk = (double)R.bk(i);
        if (i > 0) {
            const double d = (double)R.dl(i);
            if (M & XH_K0) {
                s.v[XS_K0] = fma(d * d, s.v[XS_B2], s.v[XS_K0]);
            }
            if (M & XH_K1) {
                s.v[XS_K1] = fma(d * 2, s.v[XS_BD], s.v[XS_K1]);
            }
            if (M & XH_W) {
                s.v[XS_W] = fma(d, s.v[XS_VB], s.v[XS_W]);
            }
            if (M & XH_BD) {
                s.v[XS_BD] = fma(d, s.v[XS_B2], s.v[XS_BD]);
            }
        }
        if (M & XH_B2) {
            s.v[XS_B2] = fma(bk, bk, s.v[XS_B2]);
        }
        if (M & XH_VB) {
            s.v[XS_VB] = fma((double)R.yk(i), bk, s.v[XS_VB]);
        }
    }
}

// Level 1: guesses (sums of the chunk's terms) and speculative runs of b2, vb.
// A level's records go to c[0], c[cs], c[2 cs] (one per chain).
XC_HD void xh_guess1(const XhRows &R, int i0, int i1, double *g)
{
    XcGuess b2, vb;
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        const float bk = R.bk(i);
        b2.add_product(bk, bk);
        vb.add_product(R.yk(i), bk);
    }
    g[0] = b2.value();
    g[1] = vb.value();
}

XC_HD void xh_spec1(const XhRows &R, int i0, int i1, const double *g, XcChunk *c, int cs)
{
    XcSpec sb, sv;
    sb.begin(g[0]);
    sv.begin(g[1]);
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        const double bk = (double)R.bk(i);
        sb.step(bk, bk);
        sv.step((double)R.yk(i), bk);
    }
    sb.finish(c[0], i1 <= i0);
    sv.finish(c[cs], i1 <= i0);
}

// Level 2 (chunks with i0 >= 1): bd, w, k0 from the exact b2, vb at the chunk's
// entry (b2, vb).
XC_HD void xh_guess2(const XhRows &R, int i0, int i1, double b2, double vb, double *g)
{
    XcGuess fb2, fvb, bd, w, k0;
    fb2.set(b2);
    fvb.set(vb);
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        const float bk = R.bk(i);
        if (i > 0) {
            const float d = R.dl(i);
            XcGuess db2;
            db2.add_scaled(d, fb2.hi, fb2.lo);
            bd.add_scaled(1.0f, db2.hi, db2.lo);
            k0.add_scaled(d, db2.hi, db2.lo);
            w.add_scaled(d, fvb.hi, fvb.lo);
        }
        fb2.add_product(bk, bk);
        fvb.add_product(R.yk(i), bk);
    }
    g[0] = bd.value();
    g[1] = w.value();
    g[2] = k0.value();
}

XC_HD void xh_spec2(const XhRows &R, int i0, int i1, double b2, double vb, const double *g,
                    XcChunk *c, int cs)
{
    XcSpec sbd, sw, sk0;
    sbd.begin(g[0]);
    sw.begin(g[1]);
    sk0.begin(g[2]);
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        const double bk = (double)R.bk(i);
        if (i > 0) {
            const double d = (double)R.dl(i);
            sk0.step(d * d, b2);
            sw.step(d, vb);
            sbd.step(d, b2);
        }
        b2 = fma(bk, bk, b2);
        vb = fma((double)R.yk(i), bk, vb);
    }
    const bool empty = i1 <= (i0 > 1 ? i0 : 1);
    sbd.finish(c[0], empty);
    sw.finish(c[cs], empty);
    sk0.finish(c[2 * cs], empty);
}

// Level 3 (chunks with i0 >= 1): k1 from the exact b2, bd at the chunk's entry.
XC_HD void xh_guess3(const XhRows &R, int i0, int i1, double b2, double bd, double *g)
{
    XcGuess fb2, fbd, k1;
    fb2.set(b2);
    fbd.set(bd);
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        const float bk = R.bk(i);
        if (i > 0) {
            const float d = R.dl(i);
            k1.add_scaled(2.0f * d, fbd.hi, fbd.lo);
            fbd.add_scaled(d, fb2.hi, fb2.lo);
        }
        fb2.add_product(bk, bk);
    }
    g[0] = k1.value();
}

XC_HD void xh_spec3(const XhRows &R, int i0, int i1, double b2, double bd, const double *g,
                    XcChunk *c)
{
    XcSpec sk;
    sk.begin(g[0]);
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        const double bk = (double)R.bk(i);
        if (i > 0) {
            const double d = (double)R.dl(i);
            sk.step(d * 2, bd);
            bd = fma(d, b2, bd);
        }
        b2 = fma(bk, bk, b2);
    }
    sk.finish(c[0], i1 <= (i0 > 1 ? i0 : 1));
}

// The first grid row at or after i0 (grid rows head + 1 + q min_span).
XC_HD int xh_first_grid(int i0, int head, int min_span)
{
    const int g0 = head + 1;
    return i0 <= g0 ? g0 : g0 + (i0 - g0 + min_span - 1) / min_span * min_span;
}

// Every chain through [i0, i1) from the exact entry state s; emit(q, k0, k1, w)
// at each grid row, q its index.
template <class Emit>
XC_HD void xh_output(const XhRows &R, int i0, int i1, XhState s, int head, int min_span,
                     const Emit &emit)
{
    int g = xh_first_grid(i0, head, min_span);
XC_UNROLL4
    for (int i = i0; i < i1; ++i) {
        xh_run<XH_ALL>(R, i, i + 1, s);
        if (i == g) {
            emit((g - head - 1) / min_span, s.v[XS_K0], s.v[XS_K1], s.v[XS_W]);
            g += min_span;
        }
    }
}
