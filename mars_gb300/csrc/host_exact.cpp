// The fit state's set-up on the host, in the reference's exact operation order:
// every `acc += a*b` of the reference is an explicit std::fma here, in the same
// order, and this file is compiled with -ffp-contract=off, so the results equal
// the reference's scalar (aarch64) build bit for bit.
#include "host_exact.h"

#include "error.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <thread>

#include <sched.h>

namespace mgpu {

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

void HostBasis::init(const float *X_, const float *y_, const float *w, size_t n_, size_t p_,
                     size_t ldx_)
{
    verify(!std::isfinite(NAN), "NAN check is disabled, recompile without --fast-math");
    n = n_;
    p = p_;
    ldx = ldx_;
    X = X_;
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
    b0.assign(n, 0.f);
    for (size_t i = 0; i < n; ++i) {
        yd[i] /= y_norm;
        sw[i] /= w_norm;
        y[i] = (float)yd[i];
        b0[i] = (float)sw[i];
    }
    ybo0 = 0.0;
    for (size_t i = 0; i < n; ++i) {
        ybo0 = std::fma((double)b0[i], (double)y[i], ybo0);
    }
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


}  // namespace mgpu
