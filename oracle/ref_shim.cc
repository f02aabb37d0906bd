/*
 *  ref_shim.cc -- C entry points over the reference's own MarsAlgo.
 *
 *  TEST INFRASTRUCTURE. Compiled together with the reference sources
 *  marsalgo.cc and kernels.cc (read in place, never copied) by
 *  oracle/Makefile into oracle/_ref/. It exposes the same C API as
 *  oracle/mars_oracle.c (prefix mr_ instead of mo_) so one Python wrapper
 *  drives both, and the restatement can be checked against the reference
 *  value for value.
 *
 *  The OpenMP loop below restates marslib.cc:41-148 (the pybind11 binding's
 *  parallel loop over X columns), which cannot be linked without pybind11.
 */
#include "marsalgo.h"
#include "kernels.h"

#include <omp.h>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>

#define MR_EXPORT extern "C" __attribute__((visibility("default")))

struct cov_t {
    double ff;
    double fy;
};
void argsort(int32_t *idx, const float *v, size_t n);
cov_t covariates(double *f, double *g, const float *x, const double *y,
                 double xm, double ym, double k0, float k1, size_t m);

static void set_err(char *err, size_t len, const char *msg)
{
    if (err && len) {
        snprintf(err, len, "%s", msg);
    }
}

MR_EXPORT void *mr_create(const float *X, const float *y, const float *w, size_t n, size_t p,
                          size_t max_terms, size_t ldx, char *err, size_t errlen)
{
    try {
        return new MarsAlgo(X, y, w, n, p, max_terms, ldx);
    } catch (const std::exception &e) {
        set_err(err, errlen, e.what());
        return nullptr;
    }
}

MR_EXPORT void mr_destroy(void *h) { delete static_cast<MarsAlgo *>(h); }
MR_EXPORT int mr_nbasis(void *h) { return static_cast<MarsAlgo *>(h)->nbasis(); }
MR_EXPORT int mr_nrows(void *h) { return static_cast<MarsAlgo *>(h)->nrows(); }
MR_EXPORT double mr_yvar(void *h) { return static_cast<MarsAlgo *>(h)->yvar(); }
MR_EXPORT double mr_dsse(void *h) { return static_cast<MarsAlgo *>(h)->dsse(); }

MR_EXPORT int mr_eval_all(void *h, double *lin, double *hin, double *cut, const bool *mask,
                          int rows, int mask_stride, int min_span, int end_span,
                          int linear_only, int threads, long *dgks_counter, char *err,
                          size_t errlen)
{
    (void)dgks_counter;  /* the reference's eval() takes no counter */
    MarsAlgo &algo = *static_cast<MarsAlgo *>(h);
    const int m = algo.nbasis();
    int n_procs = omp_get_num_procs();
    threads = threads <= 0 ? std::min(64, n_procs) : std::min(threads, n_procs);
    threads = std::min(threads, rows);
    if (threads < 1) {
        threads = 1;
    }
    std::atomic<bool> ok{true};
    std::string msg;
#pragma omp parallel num_threads(threads)
    {
#pragma omp for schedule(static)
        for (int i = 0; i < rows; ++i) {
            if (ok.load(std::memory_order_relaxed)) {
                try {
                    algo.eval(lin + (size_t)i * m, hin + (size_t)i * m, cut + (size_t)i * m, i,
                              mask + (size_t)i * mask_stride, min_span, end_span,
                              linear_only != 0, false);
                } catch (const std::exception &e) {
#pragma omp critical
                    {
                        if (msg.empty()) {
                            msg = e.what();
                        }
                    }
                    ok.store(false, std::memory_order_relaxed);
                }
            }
        }
    }
    if (!ok) {
        set_err(err, errlen, msg.c_str());
        return -1;
    }
    return 0;
}

MR_EXPORT double mr_append(void *h, char type, int xcol, int bcol, float hcut, int *status,
                           char *err, size_t errlen)
{
    *status = 0;
    try {
        return static_cast<MarsAlgo *>(h)->append(type, xcol, bcol, hcut);
    } catch (const std::exception &e) {
        set_err(err, errlen, e.what());
        *status = -1;
        return 0;
    }
}

MR_EXPORT void mr_argsort(int32_t *idx, const float *v, size_t n) { argsort(idx, v, n); }

MR_EXPORT void mr_covariates(double *f, double *g, const float *x, const double *y, double xm,
                             double ym, double k0, float k1, size_t m, double *ff, double *fy)
{
    cov_t o = covariates(f, g, x, y, xm, ym, k0, k1, m);
    *ff = o.ff;
    *fy = o.fy;
}

MR_EXPORT void mr_orthonormalize(size_t n, size_t m, size_t p, const float *B, size_t ldB,
                                 const float *x, const int *mask, const float *Bo, size_t ldBo,
                                 float *Bx, size_t ldBx, double *T, size_t ldT, double *s_buf,
                                 double tol, long *dgks_counter)
{
    std::atomic<long> c{0};
    mars::orthonormalize(n, m, p, B, ldB, x, mask, Bo, ldBo, Bx, ldBx, T, ldT, s_buf, tol, &c);
    if (dgks_counter) {
        *dgks_counter += c.load();
    }
}

MR_EXPORT double mr_orthonormalize_col(size_t n, size_t m, double *v, const float *Bo,
                                       size_t ldBo, double tol, long *dgks_counter)
{
    std::atomic<long> c{0};
    double w = mars::orthonormalize_col(n, m, v, Bo, ldBo, tol, &c);
    if (dgks_counter) {
        *dgks_counter += c.load();
    }
    return w;
}

MR_EXPORT double mr_dot_widen(const float *a, const float *b, size_t n)
{
    return mars::dot_widen(a, b, n);
}
