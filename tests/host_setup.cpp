// C entry for the fit's host set-up (mars_gb300/csrc/host_exact.cpp) alone, so
// the CPU tests can check it against the oracle without a GPU.
#include "host_exact.h"

#include <algorithm>
#include <cstring>
#include <exception>

extern "C" int hs_init(const float *X, const float *y, const float *w, size_t n, size_t p,
                       size_t ldx, double *yvar, double *ybo0, double *tol, float *s, float *yn,
                       float *b0, char *err, int errlen)
{
    try {
        mgpu::HostBasis hb;
        hb.init(X, y, w, n, p, ldx);
        *yvar = hb.yvar;
        *ybo0 = hb.ybo0;
        *tol = hb.tol;
        std::copy(hb.s.begin(), hb.s.end(), s);
        std::copy(hb.y.begin(), hb.y.end(), yn);
        std::copy(hb.b0.begin(), hb.b0.end(), b0);
        return 0;
    } catch (const std::exception &e) {
        std::strncpy(err, e.what(), (size_t)errlen - 1);
        err[errlen - 1] = '\0';
        return 1;
    }
}
