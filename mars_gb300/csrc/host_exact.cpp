// Host-side FP64 arithmetic in the reference's exact operation order (see
// host_exact.h for why these run on the host cores). Every `acc += a*b` of the
// reference is an explicit std::fma here, in the same order, and this file is
// compiled with -ffp-contract=off, so the results equal the reference's
// scalar (aarch64) build bit for bit.
#include "host_exact.h"

#include "error.h"
#include "xchain.cuh"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <condition_variable>
#include <cstdlib>
#include <functional>
#include <mutex>
#include <thread>

#include <sched.h>
#include <unistd.h>

namespace mgpu {

namespace {
constexpr double kDgksRatioSq = 9.0;  // kernels.h:17

// ---------------------------------------------------------------------------
// An append of a long column on several host cores. Its elementwise loops (the
// new column, the Gram-Schmidt updates v -= c q, the scalings and the row-major
// copy) split over a process-wide thread pool: memory-bound, and each element's
// value does not depend on the split. Taken for appends of at least
// MARS_GPU_HOST_PAR_ROWS rows (default 262,144) when the pool is free; shorter
// columns, and appends while another append holds the pool, run in order on
// the calling thread.
//
// The serial FP64 chains (the dot products and norms) of those appends run
// chunked with the exact speculation of xchain.cuh (guesses from plain FP64
// partial sums, XC_RUNS + 1 speculative runs per chunk of ~2,048 rows, an
// in-order walk) unless MARS_GPU_HOST_XCHAIN=0. On the 16 Grace cores of a
// GB300 machine that halves an append of 10^6 rows (41 -> 20 ms at 13 basis
// columns, 111 -> 53 ms at 50); on eight x86 cores it gained 5 %. Either way
// the results are the same bit for bit.
// ---------------------------------------------------------------------------

// A process-wide pool of host threads. The caller takes part as worker 0; idle
// workers spin briefly on the job counter, then sleep.
class HostPool {
  public:
    explicit HostPool(int nt) : nt_(nt)
    {
        for (int w = 1; w < nt_; ++w) {
            th_.emplace_back([this, w] { loop(w); });
        }
    }
    int size() const { return nt_; }
    // fn(w) for w = 0 .. size() - 1; returns when every worker has finished.
    void run(const std::function<void(int)> &fn)
    {
        job_ = &fn;
        pending_.store(nt_ - 1, std::memory_order_relaxed);
        {
            std::lock_guard<std::mutex> lk(mu_);
            epoch_.fetch_add(1, std::memory_order_release);
        }
        cv_.notify_all();
        fn(0);
        // the workers usually finish within microseconds of the caller; past
        // a short spin, give the core away so a descheduled worker can run
        for (int spin = 0; pending_.load(std::memory_order_acquire) != 0; ++spin) {
            if (spin >= 1024) {
                std::this_thread::yield();
            }
        }
    }

  private:
    void loop(int w)
    {
        unsigned seen = 0;
        for (;;) {
            unsigned e = epoch_.load(std::memory_order_acquire);
            for (int spin = 0; e == seen && spin < (1 << 16); ++spin) {
                if (spin >= 1024) {
                    std::this_thread::yield();
                }
                e = epoch_.load(std::memory_order_acquire);
            }
            if (e == seen) {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return epoch_.load(std::memory_order_acquire) != seen; });
                e = epoch_.load(std::memory_order_acquire);
            }
            seen = e;
            (*job_)(w);
            pending_.fetch_sub(1, std::memory_order_acq_rel);
        }
    }
    int nt_;
    std::vector<std::thread> th_;
    std::atomic<unsigned> epoch_{0};
    std::atomic<int> pending_{0};
    const std::function<void(int)> *job_ = nullptr;
    std::mutex mu_;
    std::condition_variable cv_;
};

std::mutex g_pool_use;  // one append at a time uses the pool

}  // namespace

// Cores this process may run on: its CPU affinity mask (which a cgroup or
// taskset narrows), else the hardware thread count.
int usable_cores()
{
    cpu_set_t set;
    CPU_ZERO(&set);
    if (sched_getaffinity(0, sizeof(set), &set) == 0) {
        const int c = CPU_COUNT(&set);
        if (c > 0) {
            return c;
        }
    }
    return (int)std::max(1u, std::thread::hardware_concurrency());
}

namespace {

// The pool of this process (none in a child forked after it was made: the
// child has no worker threads).
HostPool *host_pool()
{
    static const pid_t owner = getpid();
    static HostPool *pool = [] {
        const int nt = std::min(16, usable_cores());
        return nt > 1 ? new HostPool(nt) : nullptr;  // lives until the process exits
    }();
    return getpid() == owner ? pool : nullptr;
}

size_t host_par_rows()
{
    const char *v = std::getenv("MARS_GPU_HOST_PAR_ROWS");
    return v && *v ? (size_t)std::strtoull(v, nullptr, 10) : (size_t)262144;
}

bool host_xchain()
{
    const char *v = std::getenv("MARS_GPU_HOST_XCHAIN");
    return !(v && *v == '0');
}

// Runs the append's loops in order (pool == nullptr) or over the pool.
struct Par {
    HostPool *pool = nullptr;
    bool chunked_chains = false;

    // fn(i0, i1) over [0, n) in pieces; elementwise work only.
    template <class F>
    void rows(size_t n, const F &fn) const
    {
        if (!pool) {
            fn((size_t)0, n);
            return;
        }
        const size_t T = (size_t)pool->size(), L = (n + T - 1) / T;
        pool->run([&](int w) {
            const size_t i0 = std::min(n, (size_t)w * L), i1 = std::min(n, i0 + L);
            if (i0 < i1) {
                fn(i0, i1);
            }
        });
    }

    // acc = fma(x_i, y_i, acc) over i = 0 .. n-1 in order, from 0; term(i, x, y)
    // gives row i's FP64 factors. Chunks of ~2,048 rows (a signed chain then
    // rarely leaves its binade inside one), a contiguous range of them per thread.
    template <class Term>
    double chain(size_t n, const Term &term) const
    {
        auto run_in_order = [&](size_t i0, size_t i1, double t) {
            for (size_t i = i0; i < i1; ++i) {
                double x, y;
                term(i, x, y);
                t = std::fma(x, y, t);
            }
            return t;
        };
        if (!pool || !chunked_chains) {
            return run_in_order(0, n, 0.0);
        }
        constexpr size_t kRows = 2048;
        const int T = pool->size();
        const size_t C = std::max<size_t>((size_t)T, (n + kRows - 1) / kRows);
        const size_t L = (n + C - 1) / C, per = (C + T - 1) / T;
        static std::vector<XcChunk> rec;  // used under the pool lock only
        static std::vector<double> guess;
        rec.resize(C);
        guess.resize(C);
        double end0 = 0.0;
        auto lo = [&](size_t c) { return std::min(n, c * L); };
        auto hi = [&](size_t c) { return std::min(n, lo(c) + L); };
        pool->run([&](int w) {  // chunk sums, eight partial sums each
            for (size_t c = (size_t)w * per; c < std::min(C, (size_t)(w + 1) * per); ++c) {
                double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                size_t i = lo(c);
                for (; i + 8 <= hi(c); i += 8) {
                    for (int k = 0; k < 8; ++k) {
                        double x, y;
                        term(i + k, x, y);
                        s[k] += x * y;
                    }
                }
                for (; i < hi(c); ++i) {
                    double x, y;
                    term(i, x, y);
                    s[0] += x * y;
                }
                guess[c] = ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
            }
        });
        double pre = 0.0;
        for (size_t c = 0; c < C; ++c) {
            const double v = guess[c];
            guess[c] = pre;
            pre += v;
        }
        pool->run([&](int w) {
            for (size_t c = (size_t)w * per; c < std::min(C, (size_t)(w + 1) * per); ++c) {
                if (c == 0) {
                    end0 = run_in_order(lo(0), hi(0), 0.0);
                    continue;
                }
                XcSpec sp;
                sp.begin(guess[c]);
                for (size_t i = lo(c); i < hi(c); ++i) {
                    double x, y;
                    term(i, x, y);
                    sp.step(x, y);
                }
                sp.finish(rec[c], hi(c) <= lo(c));
            }
        });
        double t = end0;
        for (size_t c = 1; c < C; ++c) {
            bool redone = false;
            t = xc_resolve_with(rec[c], t, [&](double v) { return run_in_order(lo(c), hi(c), v); },
                                &redone);
        }
        return t;
    }
};

// Holds the pool for one append when its columns are long enough.
struct ParScope {
    Par par;
    bool held = false;
    explicit ParScope(size_t n)
    {
        if (n >= host_par_rows() && host_pool() && g_pool_use.try_lock()) {
            held = true;
            par.pool = host_pool();
            par.chunked_chains = host_xchain();
        }
    }
    ~ParScope()
    {
        if (held) {
            g_pool_use.unlock();
        }
    }
};
}  // namespace

void HostBasis::init(const float *X_, const float *y_, const float *w, size_t n_, size_t p_,
                     size_t ldx_, size_t max_terms_)
{
    verify(!std::isfinite(NAN), "NAN check is disabled, recompile without --fast-math");
    verify(max_terms_ >= 1, "max_terms must be >= 1");
    n = n_;
    p = p_;
    ldx = ldx_;
    max_terms = max_terms_;
    X = X_;
    m = 1;
    tol = ((double)n * 0.02) * DBL_EPSILON;

    // marsalgo.cc:278-352
    std::vector<double> yd(n), sw(n);
    for (size_t i = 0; i < n; ++i) {
        double yi = (double)y_[i];
        double swi = std::sqrt((double)w[i]);
        if (!std::isfinite(yi)) {
            yi = swi = 0.0;
        }
        sw[i] = swi;
        yd[i] = yi * swi;
    }
    double y_sq = 0.0, w_sq = 0.0;
    for (size_t i = 0; i < n; ++i) {
        y_sq = std::fma(yd[i], yd[i], y_sq);
        w_sq = std::fma(sw[i], sw[i], w_sq);
    }
    const double y_norm = std::sqrt(y_sq), w_norm = std::sqrt(w_sq);
    verify(y_norm > 0.0 && w_norm > 0.0, "target Y is all zero or NANs");
    y.assign(n, 0.f);
    B.assign(n * max_terms, 0.f);
    BoC.assign(n * max_terms, 0.f);
    BoR.assign(n * max_terms, 0.f);
    for (size_t i = 0; i < n; ++i) {
        yd[i] /= y_norm;
        sw[i] /= w_norm;
        y[i] = (float)yd[i];
        B[i] = BoC[i] = BoR[i * max_terms] = (float)sw[i];
    }
    double ybo0 = 0.0;
    for (size_t i = 0; i < n; ++i) {
        ybo0 = std::fma((double)BoC[i], (double)y[i], ybo0);
    }
    ybo.assign(1, ybo0);
    double ymean_sum = 0.0;
    for (size_t i = 0; i < n; ++i) {
        ymean_sum += yd[i];
    }
    const double ymean = ymean_sum / (double)n;
    double vsum = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const double dv = yd[i] - ymean;
        vsum = std::fma(dv, dv, vsum);
    }
    yvar = vsum / (double)n;

    // marsalgo.cc:359-369, one column per thread.
    s.assign(p, 1.0f);
    std::vector<double> sq(p, 0.0);
    {
        const int nt = (int)std::max<size_t>(1, std::min<size_t>(p, (size_t)usable_cores()));
        std::atomic<size_t> next{0};
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) {
            pool.emplace_back([&] {
                for (size_t j; (j = next++) < p;) {
                    const float *xj = X + j * ldx;
                    double acc = 0.0;
                    for (size_t i = 0; i < n; ++i) {
                        acc = std::fma((double)xj[i], (double)xj[i], acc);
                    }
                    sq[j] = acc;
                }
            });
        }
        for (auto &th : pool) {
            th.join();
        }
    }
    for (size_t j = 0; j < p; ++j) {
        const double rms = std::sqrt(sq[j] / (double)n);
        verify(std::isfinite(rms), "not all columns in X are finite");
        s[j] = rms > 0.0 ? (float)(1.0 / rms) : 1.0f;
    }
}

double HostBasis::dsse() const
{
    double acc = 0.0;
    for (double v : ybo) {
        acc = std::fma(v, v, acc);
    }
    return acc;
}

namespace {

// kernels.cc:194-211 against column-major Bo (column stride n).
double mgs_project(const Par &par, size_t n, size_t m, double *v, const float *BoC)
{
    double proj = 0.0;
    for (size_t j = 0; j < m; ++j) {
        const float *q = BoC + j * n;
        const double c = par.chain(n, [&](size_t i, double &x, double &y) {
            x = (double)q[i];
            y = v[i];
        });
        par.rows(n, [&](size_t i0, size_t i1) {
            for (size_t i = i0; i < i1; ++i) {
                v[i] = std::fma(-c, (double)q[i], v[i]);
            }
        });
        proj = std::fma(c, c, proj);
    }
    return proj;
}

double sum_sq(const Par &par, const double *v, size_t n)
{
    return par.chain(n, [&](size_t i, double &x, double &y) { x = y = v[i]; });
}

}  // namespace

double HostBasis::append(char type, int xcol, int bcol, float h, long *dgks)
{
    const ParScope scope(n);
    const Par &par = scope.par;
    const float sx = s[xcol];
    const float *bp = B.data() + (size_t)bcol * n;
    const float *xp = X + (size_t)xcol * ldx;
    float *Bm = B.data() + m * n;
    std::vector<double> v(n);
    par.rows(n, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; ++i) {
            float val;
            if (type == 'l') {
                val = sx * bp[i] * xp[i];
            } else {
                const float t = (type == '+') ? xp[i] - h : h - xp[i];
                val = sx * bp[i] * ((t < 0.0f) ? 0.0f : t);
            }
            Bm[i] = val;
            v[i] = (double)val;
        }
    });
    const float raw = (float)std::sqrt(sum_sq(par, v.data(), n));
    par.rows(n, [&](size_t i0, size_t i1) {
        for (size_t i = i0; i < i1; ++i) {
            Bm[i] /= raw;
        }
    });
    // kernels.cc:239-281
    const double proj = mgs_project(par, n, m, v.data(), BoC.data());
    double vn = sum_sq(par, v.data(), n);
    if (vn > tol && vn * kDgksRatioSq < proj) {
        if (dgks) {
            ++*dgks;
        }
        mgs_project(par, n, m, v.data(), BoC.data());
        vn = sum_sq(par, v.data(), n);
    }
    const double wn = std::sqrt(vn);
    if (wn * wn > tol) {
        float *q = BoC.data() + m * n;
        par.rows(n, [&](size_t i0, size_t i1) {
            for (size_t i = i0; i < i1; ++i) {
                v[i] /= wn;
                q[i] = (float)v[i];
            }
        });
        double ybo_m = par.chain(n, [&](size_t i, double &x, double &y) {
            x = (double)q[i];
            y = (double)this->y[i];
        });
        double ybo_sq = ybo_m * ybo_m;
        for (double e : ybo) {
            ybo_sq = std::fma(e, e, ybo_sq);
        }
        const double mse = (1. - ybo_sq) / (double)n;
        if (mse >= -tol) {
            par.rows(n, [&](size_t i0, size_t i1) {
                for (size_t i = i0; i < i1; ++i) {
                    BoR[i * max_terms + m] = q[i];
                }
            });
            ybo.push_back(ybo_m);
            m += 1;
            return mse < 0.0 ? 0.0 : mse;
        }
    }
    return -1.0;
}

namespace {

// The reference's projection of one candidate column (kernels.cc:327-377):
// T = Bo^T bx (rows outermost), then bx <- f32(bx - Bo T) row by row with the
// projection as a fused chain over k, and s = ||bx||^2 of the stored values.
// Eight rows are interleaved to keep the host's FMA pipes busy; each row's
// chain is unchanged.
double project_once(const HostBasis &hb, float *bx, double *T)
{
    const size_t n = hb.n, m = hb.m, ld = hb.max_terms;
    const float *Bo = hb.BoR.data();
    std::fill(T, T + m, 0.0);
    for (size_t i = 0; i < n; ++i) {
        const float *row = Bo + i * ld;
        const double xi = (double)bx[i];
        for (size_t k = 0; k < m; ++k) {
            T[k] = std::fma((double)row[k], xi, T[k]);
        }
    }
    double s = 0.0;
    size_t i = 0;
    constexpr int R = 8;
    for (; i + R <= n; i += R) {
        double pr[R] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (size_t k = 0; k < m; ++k) {
            const double t = T[k];
            for (int r = 0; r < R; ++r) {
                pr[r] = std::fma((double)Bo[(i + r) * ld + k], t, pr[r]);
            }
        }
        for (int r = 0; r < R; ++r) {
            const float vf = (float)((double)bx[i + r] - pr[r]);
            bx[i + r] = vf;
            s = std::fma((double)vf, (double)vf, s);
        }
    }
    for (; i < n; ++i) {
        double pr = 0.0;
        for (size_t k = 0; k < m; ++k) {
            pr = std::fma((double)Bo[i * ld + k], T[k], pr);
        }
        const float vf = (float)((double)bx[i] - pr);
        bx[i] = vf;
        s = std::fma((double)vf, (double)vf, s);
    }
    return s;
}

}  // namespace

ExactResult exact_candidate(const HostBasis &hb, int xcol, int bcol, const int32_t *perm,
                            int min_span, int head, int tail)
{
    const size_t n = hb.n, m = hb.m, ld = hb.max_terms;
    ExactResult r;
    std::vector<float> x(n), bx(n);
    std::vector<double> T(m + 1), T2(m + 1);
    const float *xc = hb.X + (size_t)xcol * hb.ldx;
    const float sx = hb.s[xcol];
    const float *b = hb.B.data() + (size_t)bcol * n;
    for (size_t i = 0; i < n; ++i) {
        x[i] = xc[i] * sx;
        bx[i] = b[i] * x[i];
    }
    double s = project_once(hb, bx.data(), T.data());
    double tn = 0.0;
    for (size_t k = 0; k < m; ++k) {
        tn = std::fma(T[k], T[k], tn);
    }
    if (s > hb.tol && s * kDgksRatioSq < tn) {
        r.dgks = true;
        s = project_once(hb, bx.data(), T2.data());
    }
    const float scale = (s > hb.tol) ? (float)(1.0 / std::sqrt(s + hb.tol)) : 0.0f;
    double ybx = 0.0;
    for (size_t i = 0; i < n; ++i) {
        bx[i] *= scale;
        ybx = std::fma((double)bx[i], (double)hb.y[i], ybx);
    }
    r.ybx = ybx;
    if (!perm || tail <= 0) {
        return r;
    }

    // marsalgo.cc:576-649
    const int32_t *k = perm;
    const double *ybo = hb.ybo.data();
    const float *Bo = hb.BoR.data();
    const double tol = hb.tol;
    std::vector<double> f(m + 1, 0.0), g(m + 1, 0.0);
    auto step = [&](const float *row, double xm, double ym, double k0, double k1d,
                    bool need, double &ff, double &fy) {
        for (size_t c = 0; c < m; ++c) {
            f[c] = std::fma(k0, g[c], f[c]);
            g[c] = std::fma(k1d, (double)row[c], g[c]);
        }
        f[m] = std::fma(k0, g[m], f[m]);
        g[m] = std::fma(k1d, xm, g[m]);
        if (need) {
            double a = 0.0, c2 = 0.0;
            for (size_t c = 0; c < m; ++c) {
                a = std::fma(f[c], f[c], a);
                c2 = std::fma(f[c], ybo[c], c2);
            }
            a = std::fma(f[m], f[m], a);
            c2 = std::fma(f[m], ym, c2);
            ff = a;
            fy = c2;
        }
    };
    double b_k = b[k[0]], bx_k = bx[k[0]], y_k = hb.y[k[0]];
    double ff = 0.0, fy = 0.0;
    step(Bo + (size_t)k[0] * ld, bx_k, ybx, 0.0, (double)(float)b_k, false, ff, fy);
    double k0 = 0, k1 = 0, w = 0, bd = 0;
    double vb = b_k * y_k;
    double b2 = b_k * b_k;
    size_t next_grid = (size_t)head + 1;
    double best = 0.0;
    // The rows are visited in sorted order, i.e. at random in memory: fetch
    // the ones PF steps ahead so that their misses overlap.
    constexpr size_t PF = 16;
    for (size_t i = 1; i < (size_t)tail; ++i) {
        if (i + PF < (size_t)tail) {
            const size_t kp = (size_t)k[i + PF];
            __builtin_prefetch(Bo + kp * ld);
            __builtin_prefetch(Bo + kp * ld + 16);
            __builtin_prefetch(b + kp);
            __builtin_prefetch(bx.data() + kp);
            __builtin_prefetch(hb.y.data() + kp);
            __builtin_prefetch(x.data() + kp);
        }
        b_k = b[k[i]];
        bx_k = bx[k[i]];
        y_k = hb.y[k[i]];
        const double di = (double)(float)(x[k[i - 1]] - x[k[i]]);
        const bool on_grid = (i == next_grid);
        if (on_grid) {
            next_grid += (size_t)min_span;
        }
        step(Bo + (size_t)k[i] * ld, bx_k, ybx, di, (double)(float)b_k, on_grid, ff, fy);
        k0 = std::fma(di * di, b2, k0);
        k1 = std::fma(di * 2, bd, k1);
        w = std::fma(di, vb, w);
        bd = std::fma(di, b2, bd);
        b2 = std::fma(b_k, b_k, b2);
        vb = std::fma(y_k, b_k, vb);
        if (on_grid) {
            const double uw = fy - w;
            const double den = (k0 + k1) - ff;
            const double sse = den > tol ? (uw * uw) / (den + tol) : 0;
            if (sse > best) {
                best = sse;
                r.hinge_pos = (int)i;
            }
        }
    }
    r.hinge_sse = best;
    r.hinge_row = r.hinge_pos >= 0 ? k[r.hinge_pos] : -1;
    return r;
}

void exact_candidates(const HostBasis &hb, const std::vector<int> &xcol,
                      const std::vector<int> &bcol, const std::vector<const int32_t *> &perm,
                      int min_span, int head, int tail, std::vector<ExactResult> &out,
                      int threads)
{
    const size_t cnt = xcol.size();
    out.assign(cnt, ExactResult());
    if (cnt == 0) {
        return;
    }
    const int nt = std::max(1, std::min<int>(threads, (int)cnt));
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) {
        pool.emplace_back([&] {
            for (size_t q; (q = next++) < cnt;) {
                out[q] = exact_candidate(hb, xcol[q], bcol[q], perm[q], min_span, head, tail);
            }
        });
    }
    for (auto &th : pool) {
        th.join();
    }
}

}  // namespace mgpu
