// Host build of the chunked exact accumulations (mars_gb300/csrc/xchain.cuh,
// xhinge.cuh) for the CPU tests: the routines the kernels run, in the kernels
// chunk layout and phase order, against the recurrences run in order.
#include "../mars_gb300/csrc/xhinge.cuh"

#include <functional>
#include <type_traits>
#include <vector>

namespace {
struct Term {
    const float *a, *b;
    void operator()(int i, float &x, float &y) const
    {
        x = a[i];
        y = b[i];
    }
};
// Terms with a double second factor (the append's Gram-Schmidt chains: an f32
// basis value times the f64 working column).
struct TermD {
    const float *a;
    const double *b;
};

double run_d(const TermD &t, int i0, int i1, double acc)
{
    for (int i = i0; i < i1; ++i) {
        acc = fma((double)t.a[i], t.b[i], acc);
    }
    return acc;
}
}  // namespace

// The append kernel's composition: chunk records (XC_RUNS residues) composed
// per 8 chunks and per 4 of those (XC_RUNS residues), then per 8 into block
// records and per 16 blocks into group records (RB residues each), and the
// final walk over the groups with descents down to re-running rows.
template <int RB>
double kernel_composed_impl(const float *a, const double *b, int n, int K, int *redone,
                            int *descents)
{
    const TermD term{a, b};
    const int L = n > 0 ? (n + K - 1) / K : 0;
    auto lo = [&](int c) { return c * L < n ? c * L : n; };
    auto hi = [&](int c) { return lo(c) + L < n ? lo(c) + L : n; };
    std::vector<XcRec> ch(K);
    double pre = 0.0;
    for (int c = 0; c < K; ++c) {
        XcGuess g;
        for (int i = lo(c); i < hi(c); ++i) {
            const float vh = (float)b[i];
            g.add_scaled(a[i], vh, (float)(b[i] - (double)vh));
        }
        XcSpecR sp;
        sp.begin(pre, pre == 0.0);
        for (int i = lo(c); i < hi(c); ++i) {
            sp.step((double)a[i], b[i]);
        }
        sp.finish(ch[c], hi(c) <= lo(c));
        pre += g.value();
    }
    auto rows = [&](int c, double &t, XcTrack &tr) {
        xc_run_track([&](int i, double &x, double &y) {
            x = (double)a[i];
            y = b[i];
        }, lo(c), hi(c), t, tr);
    };
    const int NS = (K + 7) / 8, NW = (NS + 3) / 4, NB = (NW + 7) / 8, NG = (NB + 15) / 16;
    std::vector<XcRec> sub(NS), warp(NW);
    std::vector<XcRecT<RB>> blk(NB), grp(NG);
    auto cnt = [](int total, int g, int F) { return total - g * F < F ? total - g * F : F; };
    auto thr_sub = [&](int s, double &t, XcTrack &tr) {
        t = xc_walk([&](int k) -> const XcRec & { return ch[s * 8 + k]; }, cnt(K, s, 8), t, tr,
                    [&](int k, double &u, XcTrack &tq) { rows(s * 8 + k, u, tq); });
    };
    auto thr_warp = [&](int w, double &t, XcTrack &tr) {
        t = xc_walk([&](int k) -> const XcRec & { return sub[w * 4 + k]; }, cnt(NS, w, 4), t, tr,
                    [&](int k, double &u, XcTrack &tq) { thr_sub(w * 4 + k, u, tq); });
    };
    auto thr_blk = [&](int bk, double &t, XcTrack &tr) {
        t = xc_walk([&](int k) -> const XcRec & { return warp[bk * 8 + k]; }, cnt(NW, bk, 8), t,
                    tr, [&](int k, double &u, XcTrack &tq) { thr_warp(bk * 8 + k, u, tq); });
    };
    for (int s = 0; s < NS; ++s) {
        for (int lane = 0; lane <= XC_RUNS; ++lane) {
            xc_compose_lane([&](int k) -> const XcRec & { return ch[s * 8 + k]; }, cnt(K, s, 8),
                            lane, [&](int k, double &u, XcTrack &tq) { rows(s * 8 + k, u, tq); },
                            sub[s]);
        }
    }
    for (int w = 0; w < NW; ++w) {
        for (int lane = 0; lane <= XC_RUNS; ++lane) {
            xc_compose_lane([&](int k) -> const XcRec & { return sub[w * 4 + k]; }, cnt(NS, w, 4),
                            lane, [&](int k, double &u, XcTrack &tq) { thr_sub(w * 4 + k, u, tq); },
                            warp[w]);
        }
    }
    for (int bk = 0; bk < NB; ++bk) {
        for (int lane = 0; lane <= RB; ++lane) {
            xc_compose_lane([&](int k) -> const XcRec & { return warp[bk * 8 + k]; },
                            cnt(NW, bk, 8), lane,
                            [&](int k, double &u, XcTrack &tq) { thr_warp(bk * 8 + k, u, tq); },
                            blk[bk]);
        }
    }
    for (int g = 0; g < NG; ++g) {
        for (int lane = 0; lane <= RB; ++lane) {  // the kernel's group lanes give up on a block
            xc_compose_lane([&](int k) -> const XcRecT<RB> & { return blk[g * 16 + k]; },
                            cnt(NB, g, 16), lane, [&](int, double &, XcTrack &tq) { tq.lost = true; },
                            grp[g]);
        }
    }
    int nre = 0, nde = 0;
    XcTrack tr;
    tr.init(0u);
    double t = 0.0;
    for (int g = 0; g < NG; ++g) {
        if (xc_track(grp[g], t, tr)) {
            continue;
        }
        for (int k = 0; k < cnt(NB, g, 16); ++k) {
            const int bk = g * 16 + k;
            if (xc_track(blk[bk], t, tr)) {
                continue;
            }
            ++nde;
            t = xc_walk([&](int w) -> const XcRec & { return warp[bk * 8 + w]; }, cnt(NW, bk, 8), t,
                        tr, [&](int w, double &u, XcTrack &tq) {
                            u = xc_walk([&](int q) -> const XcRec & { return sub[(bk * 8 + w) * 4 + q]; },
                                        cnt(NS, bk * 8 + w, 4), u, tq,
                                        [&](int q, double &z, XcTrack &tz) {
                                            const int sg = (bk * 8 + w) * 4 + q;
                                            z = xc_walk([&](int r) -> const XcRec & { return ch[sg * 8 + r]; },
                                                        cnt(K, sg, 8), z, tz,
                                                        [&](int r, double &e, XcTrack &te) {
                                                            ++nre;
                                                            rows(sg * 8 + r, e, te);
                                                        });
                                        });
                        });
        }
    }
    if (redone) {
        *redone = nre;
    }
    if (descents) {
        *descents = nde;
    }
    return t;
}

extern "C" {

double xc_host_sequential_d(const float *a, const double *b, int n)
{
    return run_d(TermD{a, b}, 0, n, 0.0);
}

// The composed form: K chunk records (XcSpecR) composed level by level with the
// fan-outs fan[0 .. nlev-1] (xc_compose_lane, one call per lane), then the top
// level walked from 0 with descents into the sub-records where a record cannot
// vouch for its entry, and the rows of a chunk re-run in order at the bottom.
// guess_mode as in xc_host_chunked. *redone counts the chunks the final walk
// re-ran, *descents the composite records it could not take as they are;
// built[0..1] the same counts while the levels were composed.
double xc_host_composed(const float *a, const double *b, int n, int K, const int *fan, int nlev,
                        int guess_mode, double scale, int *redone, int *descents, int *built)
{
    const TermD term{a, b};
    const int L = n > 0 ? (n + K - 1) / K : 0;
    auto lo = [&](int c) { return c * L < n ? c * L : n; };
    auto hi = [&](int c) { return lo(c) + L < n ? lo(c) + L : n; };
    std::vector<double> sums(K);
    for (int c = 0; c < K; ++c) {
        XcGuess g;
        for (int i = lo(c); i < hi(c); ++i) {
            const float vh = (float)b[i];
            g.add_scaled(a[i], vh, (float)(b[i] - (double)vh));
        }
        sums[c] = g.value();
    }
    std::vector<std::vector<XcRec>> lev(1, std::vector<XcRec>(K));
    lev.reserve(nlev + 1);
    double pre = 0.0, tru = 0.0;
    for (int c = 0; c < K; ++c) {
        double guess = pre;
        if (guess_mode == 1) {
            guess = pre * (1.0 + scale);
        } else if (guess_mode == 2) {
            const uint32_t E = (xc_hi(tru) >> 20) & 0x7ffu;
            const double u = E > 52u ? xc_words((E - 52u) << 20, 0u) : 0.0;
            guess = tru + scale * u;
        } else if (guess_mode == 3) {
            guess = scale;
        }
        XcSpecR sp;
        sp.begin(guess, guess == 0.0);
        for (int i = lo(c); i < hi(c); ++i) {
            sp.step((double)a[i], b[i]);
        }
        sp.finish(lev[0][c], hi(c) <= lo(c));
        pre += sums[c];
        tru = run_d(term, lo(c), hi(c), tru);
    }
    int nre = 0, nde = 0;
    // through(l, k, t, tr): across record k of level l another way
    std::function<void(int, int, double &, XcTrack &)> through = [&](int l, int k, double &t,
                                                                     XcTrack &tr) {
        if (l == 0) {
            ++nre;
            xc_run_track([&](int i, double &x, double &y) {
                x = (double)a[i];
                y = b[i];
            }, lo(k), hi(k), t, tr);
            return;
        }
        ++nde;
        const int F = fan[l - 1], c0 = k * F, sz = (int)lev[l - 1].size();
        t = xc_walk([&](int q) -> const XcRec & { return lev[l - 1][c0 + q]; },
                    sz - c0 < F ? sz - c0 : F, t, tr,
                    [&](int q, double &v, XcTrack &tq) { through(l - 1, c0 + q, v, tq); });
    };
    for (int l = 0; l < nlev; ++l) {
        const std::vector<XcRec> &sub = lev.back();
        const int F = fan[l], G = ((int)sub.size() + F - 1) / F;
        std::vector<XcRec> up(G);
        for (int g = 0; g < G; ++g) {
            const int c0 = g * F, cnt = (int)sub.size() - c0 < F ? (int)sub.size() - c0 : F;
            for (int lane = 0; lane <= XC_RUNS; ++lane) {
                xc_compose_lane([&](int k) -> const XcRec & { return sub[c0 + k]; }, cnt, lane,
                                [&](int k, double &v, XcTrack &tq) { through(l, c0 + k, v, tq); },
                                up[g]);
            }
        }
        lev.push_back(up);
    }
    const int built_re = nre, built_de = nde;
    nre = nde = 0;
    XcTrack tr;
    tr.init(0u);
    const double t = xc_walk([&](int k) -> const XcRec & { return lev[nlev][k]; },
                             (int)lev[nlev].size(), 0.0, tr,
                             [&](int k, double &v, XcTrack &tq) { through(nlev, k, v, tq); });
    if (built) {
        built[0] = built_re;
        built[1] = built_de;
    }
    if (redone) {
        *redone = nre;
    }
    if (descents) {
        *descents = nde;
    }
    return t;
}

// The append kernel's levels with 4 or 8 residues at the block and group levels.
double xc_host_kernel4(const float *a, const double *b, int n, int K, int *redone, int *descents)
{
    return kernel_composed_impl<4>(a, b, n, K, redone, descents);
}
double xc_host_kernel8(const float *a, const double *b, int n, int K, int *redone, int *descents)
{
    return kernel_composed_impl<8>(a, b, n, K, redone, descents);
}

// The recurrence as written.
double xc_host_sequential(const float *a, const float *b, int n)
{
    return xc_run(Term{a, b}, 0, n, 0.0);
}

// K chunks of ceil(n / K) rows. guess_mode 0: float-float prefix guesses (the
// kernel's); 1: those guesses scaled by (1 + scale); 2: the true entry value
// plus `scale` ulps of it; 3: `scale` itself for every chunk. *redone counts the
// chunks re-run in order.
double xc_host_chunked(const float *a, const float *b, int n, int K, int guess_mode,
                       double scale, int *redone)
{
    const Term term{a, b};
    const int L = n > 0 ? (n + K - 1) / K : 0;
    std::vector<XcChunk> ch(K);
    std::vector<double> sums(K);
    for (int c = 0; c < K; ++c) {
        const int i0 = c * L < n ? c * L : n, i1 = i0 + L < n ? i0 + L : n;
        XcGuess g;
        for (int i = i0; i < i1; ++i) {
            g.add_product(a[i], b[i]);
        }
        sums[c] = g.value();
    }
    double pre = 0.0, tru = 0.0;
    double t0 = 0.0;
    for (int c = 0; c < K; ++c) {
        const int i0 = c * L < n ? c * L : n, i1 = i0 + L < n ? i0 + L : n;
        double guess = pre;
        if (guess_mode == 1) {
            guess = pre * (1.0 + scale);
        } else if (guess_mode == 2) {
            const uint32_t E = (xc_hi(tru) >> 20) & 0x7ffu;
            const double u = E > 52u ? xc_words((E - 52u) << 20, 0u) : 0.0;
            guess = tru + scale * u;
        } else if (guess_mode == 3) {
            guess = scale;
        }
        if (c == 0) {
            t0 = xc_run(term, i0, i1, 0.0);
        } else {
            xc_speculate(term, i0, i1, guess, ch[c]);
        }
        pre += sums[c];
        tru = xc_run(term, i0, i1, tru);
    }
    double t = t0;
    int nre = 0;
    for (int c = 1; c < K; ++c) {
        const int i0 = c * L < n ? c * L : n, i1 = i0 + L < n ? i0 + L : n;
        bool re = false;
        t = xc_resolve(term, i0, i1, ch[c], t, &re);
        nre += re ? 1 : 0;
    }
    if (redone) {
        *redone = nre;
    }
    return t;
}

// The hinge scalars in order: out[3 q + {0, 1, 2}] = k0, k1, w at grid row q.
void xh_host_sequential(const float *b, const float *y, const float *x, int tail, int head,
                        int min_span, double *out)
{
    const XhRows R{b, y, x};
    XhState s{};
    xh_output(R, 0, tail, s, head, min_span, [&](int q, double k0, double k1, double w) {
        out[3 * q] = k0;
        out[3 * q + 1] = k1;
        out[3 * q + 2] = w;
    });
}

// The phases of k_hinge_xscalars with K chunks; *redone counts re-run chunks.
void xh_host_chunked(const float *b, const float *y, const float *x, int tail, int head,
                     int min_span, int K, double *out, int *redone)
{
    const XhRows R{b, y, x};
    const int L = tail > 0 ? (tail + K - 1) / K : 0;
    auto lo = [&](int c) { return c * L < tail ? c * L : tail; };
    auto hi = [&](int c) { return lo(c) + L < tail ? lo(c) + L : tail; };
    std::vector<double> st((size_t)XS_N * K, 0.0), g(3 * (size_t)K, 0.0), gs(3 * (size_t)K);
    std::vector<XcChunk> ch(3 * (size_t)K);
    auto S = [&](int j, int c) -> double & { return st[(size_t)j * K + c]; };
    int nre = 0;
    auto prefix = [&](int nv) {
        for (int v = 0; v < nv; ++v) {
            double acc = 0.0;
            for (int c = 0; c < K; ++c) {
                gs[(size_t)v * K + c] = acc;
                acc += g[(size_t)c * 3 + v];
            }
        }
    };
    auto guess = [&](int v, int c) { return gs[(size_t)v * K + c]; };
    auto walk = [&](int j, int slot, auto rerun_mask) {
        for (int c = 1; c + 1 < K; ++c) {
            bool re = false;
            const double t = S(j, c);
            S(j, c + 1) = xc_resolve_with(ch[(size_t)slot * K + c], t, [&](double v) {
                XhState s{};
                for (int q = 0; q < XS_N; ++q) {
                    s.v[q] = S(q, c);
                }
                s.v[j] = v;
                xh_run<decltype(rerun_mask)::value>(R, lo(c), hi(c), s);
                return s.v[j];
            }, &re);
            nre += re ? 1 : 0;
        }
    };
    // level 1
    for (int c = 0; c < K; ++c) {
        xh_guess1(R, lo(c), hi(c), &g[(size_t)c * 3]);
    }
    prefix(2);
    for (int c = 0; c < K; ++c) {
        if (c == 0) {
            XhState s{};
            xh_run<XH_B2 | XH_VB>(R, lo(0), hi(0), s);
            if (K > 1) {
                S(XS_B2, 1) = s.v[XS_B2];
                S(XS_VB, 1) = s.v[XS_VB];
            }
        } else {
            const double gg[2] = {guess(0, c), guess(1, c)};
            xh_spec1(R, lo(c), hi(c), gg, &ch[c], K);
        }
    }
    walk(XS_B2, 0, std::integral_constant<int, XH_B2>());
    walk(XS_VB, 1, std::integral_constant<int, XH_VB>());
    // level 2
    for (int c = 0; c < K; ++c) {
        xh_guess2(R, lo(c), hi(c), S(XS_B2, c), S(XS_VB, c), &g[(size_t)c * 3]);
    }
    prefix(3);
    for (int c = 0; c < K; ++c) {
        if (c == 0) {
            XhState s{};
            xh_run<XH_B2 | XH_VB | XH_BD | XH_W | XH_K0>(R, lo(0), hi(0), s);
            if (K > 1) {
                S(XS_BD, 1) = s.v[XS_BD];
                S(XS_W, 1) = s.v[XS_W];
                S(XS_K0, 1) = s.v[XS_K0];
            }
        } else {
            const double gg[3] = {guess(0, c), guess(1, c), guess(2, c)};
            xh_spec2(R, lo(c), hi(c), S(XS_B2, c), S(XS_VB, c), gg, &ch[c], K);
        }
    }
    walk(XS_BD, 0, std::integral_constant<int, XH_B2 | XH_BD>());
    walk(XS_W, 1, std::integral_constant<int, XH_VB | XH_W>());
    walk(XS_K0, 2, std::integral_constant<int, XH_B2 | XH_K0>());
    // level 3
    for (int c = 0; c < K; ++c) {
        xh_guess3(R, lo(c), hi(c), S(XS_B2, c), S(XS_BD, c), &g[(size_t)c * 3]);
    }
    prefix(1);
    for (int c = 0; c < K; ++c) {
        if (c == 0) {
            XhState s{};
            xh_run<XH_B2 | XH_BD | XH_K1>(R, lo(0), hi(0), s);
            if (K > 1) {
                S(XS_K1, 1) = s.v[XS_K1];
            }
        } else {
            const double gg[1] = {guess(0, c)};
            xh_spec3(R, lo(c), hi(c), S(XS_B2, c), S(XS_BD, c), gg, &ch[c]);
        }
    }
    walk(XS_K1, 0, std::integral_constant<int, XH_B2 | XH_BD | XH_K1>());
    // output
    for (int c = 0; c < K; ++c) {
        XhState s{};
        for (int q = 0; q < XS_N; ++q) {
            s.v[q] = S(q, c);
        }
        xh_output(R, lo(c), hi(c), s, head, min_span, [&](int q, double k0, double k1, double w) {
            out[3 * q] = k0;
            out[3 * q + 1] = k1;
            out[3 * q + 2] = w;
        });
    }
    if (redone) {
        *redone = nre;
    }
}
}
