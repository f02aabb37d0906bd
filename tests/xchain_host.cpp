// Host build of the chunked exact accumulation (mars_gb300/csrc/xchain.cuh) for
// the CPU tests: the same xc_speculate / xc_resolve the kernel runs, with the
// chunk layout of the kernel, against the plain sequential recurrence.
#include "../mars_gb300/csrc/xchain.cuh"

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
}  // namespace

extern "C" {

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
}
