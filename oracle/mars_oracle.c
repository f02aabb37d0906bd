/*
 *  mars_oracle.c -- CPU restatement of the reference MARS forward pass.
 *
 *  TEST INFRASTRUCTURE. This file is the parity oracle and the timed CPU
 *  baseline. Only the test suite, the smoke check and the benchmark's CPU
 *  legs load it; the product (mars_gb300) never links or calls it.
 *
 *  It restates, in plain C with OpenMP over candidate X columns, the
 *  reference's scalar (non-AVX) code path -- the one the reference itself
 *  compiles on aarch64:
 *
 *    constructor      marsalgo.cc:266-370
 *    eval (per xcol)  marsalgo.cc:402-662
 *    covariates_impl  marsalgo.cc:91-151   (scalar branch, m0 = 0)
 *    argsort          marsalgo.cc:33-39    (stable, descending)
 *    append           marsalgo.cc:760-875
 *    orthonormalize   kernels.cc:283-417   (scalar branches)
 *    orthonormalize_col / mgs_project_col  kernels.cc:194-281
 *    dot_widen        kernels.cc:215-237
 *    OpenMP eval loop marslib.cc:41-148
 *
 *  Every `acc += a*b` of the reference is written as fma(a, b, acc): GCC
 *  contracts those expressions into fused multiply-adds by default
 *  (-ffp-contract=fast), and aarch64 defines FP_FAST_FMA, so the reference's
 *  own `fma()` calls are fused too. This file is compiled with
 *  -ffp-contract=off so that no other expression is fused behind our back.
 *  With that, the results are bit-identical to the reference built without
 *  its AVX branches (the recipe in oracle/Makefile checks exactly this).
 */
#include <float.h>
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MO_EXPORT __attribute__((visibility("default")))
#define DGKS_GATE_RATIO_SQ 9.0  /* kernels.h:17 */

typedef struct {
    size_t n, p, ldx, max_terms, m;
    const float *X;   /* borrowed, column-major, column stride ldx */
    float  *y;        /* normalised target, f32 storage (n) */
    float  *B;        /* basis, column-major n x max_terms */
    float  *Bo;       /* orthonormal basis, row-major n x max_terms */
    double *ybo;      /* Bo^T y per live column (max_terms) */
    float  *s;        /* 1/rms per X column (p) */
    double yvar, tol;
} mo_algo;

static void set_err(char *err, size_t len, const char *msg)
{
    if (err && len) {
        snprintf(err, len, "%s", msg);
    }
}

/* ------------------------------------------------------------------------ */
/*  Kernels (kernels.cc, scalar branches)                                    */
/* ------------------------------------------------------------------------ */

MO_EXPORT double mo_dot_widen(const float *a, const float *b, size_t n)
{
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) {
        s = fma((double)a[i], (double)b[i], s);
    }
    return s;
}

/* kernels.cc:56-78 (scalar): sequential fused chain over k. */
static inline double dot_bo(const float *bo_row, const double *tc, size_t m)
{
    double acc = 0.0;
    for (size_t k = 0; k < m; ++k) {
        acc = fma((double)bo_row[k], tc[k], acc);
    }
    return acc;
}

/* kernels.cc:38-52 (scalar). */
static inline void axpy_m(double *tc, const float *bo_row, double scalar, size_t m)
{
    for (size_t k = 0; k < m; ++k) {
        tc[k] = fma((double)bo_row[k], scalar, tc[k]);
    }
}

/* kernels.cc:194-211 */
static double mgs_project_col(size_t n, size_t m, double *v, const float *Bo, size_t ldBo)
{
    double proj_norm2 = 0.0;
    for (size_t j = 0; j < m; ++j) {
        double c = 0.0;
        for (size_t i = 0; i < n; ++i) {
            c = fma((double)Bo[i * ldBo + j], v[i], c);
        }
        for (size_t i = 0; i < n; ++i) {
            v[i] = fma(-c, (double)Bo[i * ldBo + j], v[i]);
        }
        proj_norm2 = fma(c, c, proj_norm2);
    }
    return proj_norm2;
}

/* kernels.cc:239-281 */
MO_EXPORT double mo_orthonormalize_col(size_t n, size_t m, double *v, const float *Bo,
                                       size_t ldBo, double tol, long *dgks_counter)
{
    const double proj_norm2 = mgs_project_col(n, m, v, Bo, ldBo);
    double v_norm2 = 0.0;
    for (size_t i = 0; i < n; ++i) {
        v_norm2 = fma(v[i], v[i], v_norm2);
    }
    if (v_norm2 > tol && v_norm2 * DGKS_GATE_RATIO_SQ < proj_norm2) {
        if (dgks_counter) {
            ++*dgks_counter;
        }
        mgs_project_col(n, m, v, Bo, ldBo);
        v_norm2 = 0.0;
        for (size_t i = 0; i < n; ++i) {
            v_norm2 = fma(v[i], v[i], v_norm2);
        }
    }
    const double w = sqrt(v_norm2);
    if (w * w > tol) {
        for (size_t i = 0; i < n; ++i) {
            v[i] /= w;
        }
    }
    return w;
}

/*
 *  kernels.cc:283-417. Bx = B[:,mask]*x, T = Bo^T Bx (f64), Bx -= Bo T with an
 *  f32 round, s = ||Bx||^2 of the rounded values, DGKS retry when
 *  9 s < ||T||^2, then Bx *= 1/sqrt(s+tol) (0 when s <= tol).
 */
MO_EXPORT void mo_orthonormalize(size_t n, size_t m, size_t p,
                                 const float *B, size_t ldB, const float *x,
                                 const int *mask, const float *Bo, size_t ldBo,
                                 float *Bx, size_t ldBx, double *T, size_t ldT,
                                 double *s_buf, double tol, long *dgks_counter)
{
    for (size_t j = 0; j < p; ++j) {
        const float *b  = B + (size_t)mask[j] * ldB;
        float       *bx = Bx + j * ldBx;
        for (size_t i = 0; i < n; ++i) {
            bx[i] = b[i] * x[i];
        }
    }

    /* Phase 1: T = Bo^T Bx, rows outermost, f64 accumulation. */
    for (size_t j = 0; j < p; ++j) {
        memset(T + j * ldT, 0, m * sizeof(double));
    }
    for (size_t i = 0; i < n; ++i) {
        const float *bo_row = Bo + i * ldBo;
        for (size_t j = 0; j < p; ++j) {
            axpy_m(T + j * ldT, bo_row, (double)Bx[i + j * ldBx], m);
        }
    }

    /* Phase 2a: subtract the projection, round to f32, norm of the stored value. */
    memset(s_buf, 0, p * sizeof(double));
    for (size_t i = 0; i < n; ++i) {
        const float *bo_row = Bo + i * ldBo;
        for (size_t j = 0; j < p; ++j) {
            float       *bx  = Bx + j * ldBx;
            const double v   = (double)bx[i] - dot_bo(bo_row, T + j * ldT, m);
            const float  v32 = (float)v;
            bx[i] = v32;
            const double vb = (double)v32;
            s_buf[j] = fma(vb, vb, s_buf[j]);
        }
    }

    /* Phase 2b: DGKS retry on the cancelling columns. */
    for (size_t j = 0; j < p; ++j) {
        double *tc = T + j * ldT;
        float  *bx = Bx + j * ldBx;
        double t_norm2 = 0.0;
        for (size_t k = 0; k < m; ++k) {
            t_norm2 = fma(tc[k], tc[k], t_norm2);
        }
        if (s_buf[j] > tol && s_buf[j] * DGKS_GATE_RATIO_SQ < t_norm2) {
            if (dgks_counter) {
                ++*dgks_counter;
            }
            memset(tc, 0, m * sizeof(double));
            for (size_t i = 0; i < n; ++i) {
                axpy_m(tc, Bo + i * ldBo, (double)bx[i], m);
            }
            double s = 0.0;
            for (size_t i = 0; i < n; ++i) {
                const double v   = (double)bx[i] - dot_bo(Bo + i * ldBo, tc, m);
                const float  v32 = (float)v;
                bx[i] = v32;
                const double vb = (double)v32;
                s = fma(vb, vb, s);
            }
            s_buf[j] = s;
        }
    }

    /* Phase 2c: normalise (f32 multiply by an f32 scale). */
    for (size_t j = 0; j < p; ++j) {
        float       *bx    = Bx + j * ldBx;
        const double s     = s_buf[j];
        const float  scale = (s > tol) ? (float)(1.0 / sqrt(s + tol)) : 0.0f;
        for (size_t i = 0; i < n; ++i) {
            bx[i] *= scale;
        }
    }
}

/* ------------------------------------------------------------------------ */
/*  Sweep helpers (marsalgo.cc)                                              */
/* ------------------------------------------------------------------------ */

typedef struct { double ff, fy; } mo_cov;

/* marsalgo.cc:91-151, scalar branch. */
static inline mo_cov covariates_impl(bool need_sse, double *f, double *g, const float *x,
                                     const double *y, double xm, double ym, double k0,
                                     float k1, size_t m)
{
    mo_cov o = {0.0, 0.0};
    const double k1d = (double)k1;
    for (size_t i = 0; i < m; ++i) {
        f[i] = fma(k0, g[i], f[i]);
        g[i] = fma(k1d, (double)x[i], g[i]);
        if (need_sse) {
            o.ff = fma(f[i], f[i], o.ff);
            o.fy = fma(f[i], y[i], o.fy);
        }
    }
    f[m] = fma(k0, g[m], f[m]);
    g[m] = fma(k1d, xm, g[m]);
    if (need_sse) {
        o.ff = fma(f[m], f[m], o.ff);
        o.fy = fma(f[m], ym, o.fy);
    }
    return o;
}

MO_EXPORT void mo_covariates(double *f, double *g, const float *x, const double *y,
                             double xm, double ym, double k0, float k1, size_t m,
                             double *ff, double *fy)
{
    mo_cov o = covariates_impl(true, f, g, x, y, xm, ym, k0, k1, m);
    *ff = o.ff;
    *fy = o.fy;
}

/*
 *  marsalgo.cc:33-39: std::stable_sort of indexes with comparator v[i] > v[j],
 *  i.e. descending by value, ties in ascending index order. Bottom-up merge
 *  sort (stable).
 */
MO_EXPORT void mo_argsort(int32_t *idx, const float *v, size_t n)
{
    int32_t *tmp = (int32_t *)malloc(n * sizeof(int32_t) + 1);
    for (size_t i = 0; i < n; ++i) {
        idx[i] = (int32_t)i;
    }
    int32_t *src = idx, *dst = tmp;
    for (size_t width = 1; width < n; width *= 2) {
        for (size_t lo = 0; lo < n; lo += 2 * width) {
            size_t mid = lo + width < n ? lo + width : n;
            size_t hi  = lo + 2 * width < n ? lo + 2 * width : n;
            size_t a = lo, b = mid, o = lo;
            while (a < mid && b < hi) {
                /* take from the right run only when strictly greater */
                if (v[src[b]] > v[src[a]]) {
                    dst[o++] = src[b++];
                } else {
                    dst[o++] = src[a++];
                }
            }
            while (a < mid) {
                dst[o++] = src[a++];
            }
            while (b < hi) {
                dst[o++] = src[b++];
            }
        }
        int32_t *t = src;
        src = dst;
        dst = t;
    }
    if (src != idx) {
        memcpy(idx, src, n * sizeof(int32_t));
    }
    free(tmp);
}

/* ------------------------------------------------------------------------ */
/*  MarsAlgo                                                                 */
/* ------------------------------------------------------------------------ */

/* marsalgo.cc:266-370 */
MO_EXPORT void *mo_create(const float *X, const float *y, const float *w, size_t n,
                          size_t p, size_t max_terms, size_t ldx, char *err, size_t errlen)
{
    if (isfinite(NAN)) {
        set_err(err, errlen, "NAN check is disabled, recompile without --fast-math");
        return NULL;
    }
    if (max_terms < 1) {
        max_terms = 1;
    }
    mo_algo *a = (mo_algo *)calloc(1, sizeof(mo_algo));
    a->n = n;
    a->p = p;
    a->ldx = ldx;
    a->max_terms = max_terms;
    a->m = 1;
    a->X = X;
    a->tol = ((double)n * 0.02) * DBL_EPSILON;
    a->y   = (float *)calloc(n ? n : 1, sizeof(float));
    a->B   = (float *)calloc(n * max_terms + 1, sizeof(float));
    a->Bo  = (float *)calloc(n * max_terms + 1, sizeof(float));
    a->ybo = (double *)calloc(max_terms + 1, sizeof(double));
    a->s   = (float *)calloc(p + 1, sizeof(float));
    double *yd = (double *)malloc((n + 1) * sizeof(double));
    double *sw = (double *)malloc((n + 1) * sizeof(double));

    for (size_t i = 0; i < n; ++i) {
        double yi  = (double)y[i];
        double swi = sqrt((double)w[i]);
        if (!isfinite(yi)) {
            yi = swi = 0.0;
        }
        sw[i] = swi;
        yd[i] = yi * swi;
    }
    double y_sq = 0.0, w_sq = 0.0;
    for (size_t i = 0; i < n; ++i) {
        y_sq = fma(yd[i], yd[i], y_sq);
        w_sq = fma(sw[i], sw[i], w_sq);
    }
    const double y_norm = sqrt(y_sq);
    const double w_norm = sqrt(w_sq);
    if (!(y_norm > 0.0 && w_norm > 0.0)) {
        set_err(err, errlen, "target Y is all zero or NANs");
        goto fail;
    }
    for (size_t i = 0; i < n; ++i) {
        yd[i] /= y_norm;
        sw[i] /= w_norm;
    }
    for (size_t i = 0; i < n; ++i) {
        a->y[i] = (float)yd[i];
    }
    for (size_t i = 0; i < n; ++i) {
        a->B[i] = a->Bo[i * max_terms] = (float)sw[i];
    }
    {
        double ybo0 = 0.0;
        for (size_t i = 0; i < n; ++i) {
            ybo0 = fma((double)a->Bo[i * max_terms], (double)a->y[i], ybo0);
        }
        a->ybo[0] = ybo0;
    }
    {
        double ymean_sum = 0.0;
        for (size_t i = 0; i < n; ++i) {
            ymean_sum += yd[i];
        }
        const double ymean = ymean_sum / (double)n;
        double vsum = 0.0;
        for (size_t i = 0; i < n; ++i) {
            const double dv = yd[i] - ymean;
            vsum = fma(dv, dv, vsum);
        }
        a->yvar = vsum / (double)n;
    }
    for (size_t j = 0; j < p; ++j) {
        const float *xj = X + j * ldx;
        double sq = 0.0;
        for (size_t i = 0; i < n; ++i) {
            sq = fma((double)xj[i], (double)xj[i], sq);
        }
        const double rms = sqrt(sq / (double)n);
        if (!isfinite(rms)) {
            set_err(err, errlen, "not all columns in X are finite");
            goto fail;
        }
        a->s[j] = rms > 0.0 ? (float)(1.0 / rms) : 1.0f;
    }
    free(yd);
    free(sw);
    return a;
fail:
    free(yd);
    free(sw);
    free(a->y);
    free(a->B);
    free(a->Bo);
    free(a->ybo);
    free(a->s);
    free(a);
    return NULL;
}

MO_EXPORT void mo_destroy(void *h)
{
    mo_algo *a = (mo_algo *)h;
    if (!a) {
        return;
    }
    free(a->y);
    free(a->B);
    free(a->Bo);
    free(a->ybo);
    free(a->s);
    free(a);
}

MO_EXPORT int mo_nbasis(void *h) { return (int)((mo_algo *)h)->m; }
MO_EXPORT int mo_nrows(void *h) { return (int)((mo_algo *)h)->n; }
MO_EXPORT double mo_yvar(void *h) { return ((mo_algo *)h)->yvar; }
MO_EXPORT double mo_tol(void *h) { return ((mo_algo *)h)->tol; }

/* marsalgo.cc:389-396 */
MO_EXPORT double mo_dsse(void *h)
{
    mo_algo *a = (mo_algo *)h;
    double s = 0.0;
    for (size_t j = 0; j < a->m; ++j) {
        s = fma(a->ybo[j], a->ybo[j], s);
    }
    return s;
}

/* Copies of the device-independent state, for tests. */
MO_EXPORT void mo_get_state(void *h, float *y, float *B, float *Bo, double *ybo, float *s)
{
    mo_algo *a = (mo_algo *)h;
    if (y) memcpy(y, a->y, a->n * sizeof(float));
    if (B) memcpy(B, a->B, a->n * a->max_terms * sizeof(float));
    if (Bo) memcpy(Bo, a->Bo, a->n * a->max_terms * sizeof(float));
    if (ybo) memcpy(ybo, a->ybo, a->max_terms * sizeof(double));
    if (s) memcpy(s, a->s, a->p * sizeof(float));
}

/* Per-thread working memory for eval (marsalgo.cc:223-264). */
typedef struct {
    float   *x, *d, *Bx;
    int32_t *k;
    double  *f, *g, *ybx, *hsse, *T;
    int     *bcols, *hidx;
} mo_scratch;

static void scratch_alloc(mo_scratch *S, size_t n, size_t cap)
{
    S->x     = (float *)malloc((n + 1) * sizeof(float));
    S->d     = (float *)malloc((n + 1) * sizeof(float));
    S->k     = (int32_t *)malloc((n + 1) * sizeof(int32_t));
    S->Bx    = (float *)malloc((n * cap + 1) * sizeof(float));
    S->f     = (double *)malloc((cap + 2) * sizeof(double));
    S->g     = (double *)malloc((cap + 2) * sizeof(double));
    S->ybx   = (double *)malloc((cap + 1) * sizeof(double));
    S->hsse  = (double *)malloc((cap + 1) * sizeof(double));
    S->T     = (double *)malloc((cap * cap + 1) * sizeof(double));
    S->bcols = (int *)malloc((cap + 1) * sizeof(int));
    S->hidx  = (int *)malloc((cap + 1) * sizeof(int));
}

static void scratch_free(mo_scratch *S)
{
    free(S->x); free(S->d); free(S->k); free(S->Bx); free(S->f); free(S->g);
    free(S->ybx); free(S->hsse); free(S->T); free(S->bcols); free(S->hidx);
}

/*
 *  marsalgo.cc:402-662. One candidate X column against every masked parent.
 *  Returns 0, or -1 with a message for an invalid argument.
 */
static int eval_one(mo_algo *a, mo_scratch *S, double *linear_dsse, double *hinge_dsse,
                    double *hinge_cuts, int xcol, const bool *bmask, int min_span,
                    int end_span, bool linear_only, long *dgks_counter, char *err,
                    size_t errlen)
{
    if (!(xcol >= 0 && (size_t)xcol < a->p)) {
        set_err(err, errlen, "invalid X column index");
        return -1;
    }
    if (min_span < 1) {
        set_err(err, errlen, "min_span must be >= 1");
        return -1;
    }
    const size_t m = a->m, n = a->n;
    for (size_t j = 0; j < m; ++j) {
        linear_dsse[j] = 0.0;
        hinge_dsse[j]  = 0.0;
        hinge_cuts[j]  = NAN;
    }
    size_t p = 0;
    for (size_t j = 0; j < m; ++j) {
        if (bmask[j]) {
            S->bcols[p++] = (int)j;
        }
    }
    if (p == 0) {
        return 0;
    }
    const float *xc = a->X + (size_t)xcol * a->ldx;
    const float  sx = a->s[xcol];
    for (size_t i = 0; i < n; ++i) {
        S->x[i] = xc[i] * sx;
    }
    mo_orthonormalize(n, m, p, a->B, n, S->x, S->bcols, a->Bo, a->max_terms, S->Bx, n,
                      S->T, m, S->ybx, a->tol, dgks_counter);
    for (size_t j = 0; j < p; ++j) {
        S->ybx[j] = mo_dot_widen(S->Bx + j * n, a->y, n);
        linear_dsse[S->bcols[j]] = S->ybx[j] * S->ybx[j];
    }
    if (linear_only) {
        return 0;
    }
    for (size_t j = 0; j < p; ++j) {
        S->hidx[j] = -1;
        S->hsse[j] = 0.0;
    }
    mo_argsort(S->k, xc, n);
    for (size_t i = 1; i < n; ++i) {
        S->d[i] = S->x[S->k[i - 1]] - S->x[S->k[i]];
    }
    /* The reference computes tail = n - end_span in size_t; an end_span >= n
     * leaves no cut to evaluate. */
    const size_t head = (size_t)(end_span > 0 ? end_span : 0);
    const size_t tail = head < n ? n - head : 0;
    const int32_t *k = S->k;
    const float *y   = a->y;
    const double tol = a->tol;
    const size_t ldBo = a->max_terms;
    for (size_t j = 0; j < p; ++j) {
        double *f = S->f, *g = S->g;
        memset(f, 0, (m + 1) * sizeof(double));
        memset(g, 0, (m + 1) * sizeof(double));
        const float *b  = a->B + (size_t)S->bcols[j] * n;
        const float *bx = S->Bx + j * n;
        double b_k  = b[k[0]];
        double bx_k = bx[k[0]];
        double y_k  = y[k[0]];
        covariates_impl(false, f, g, a->Bo + (size_t)k[0] * ldBo, a->ybo, bx_k, S->ybx[j],
                        0, (float)b_k, m);
        double k0 = 0, k1 = 0, w = 0, bd = 0;
        double vb = b_k * y_k;
        double b2 = b_k * b_k;
        size_t next_grid = head + 1;
        for (size_t i = 1; i < tail; ++i) {
            b_k  = b[k[i]];
            bx_k = bx[k[i]];
            y_k  = y[k[i]];
            const double di = S->d[i];
            const bool on_grid = (i == next_grid);
            if (on_grid) {
                next_grid += (size_t)min_span;
            }
            const float *bo_row = a->Bo + (size_t)k[i] * ldBo;
            mo_cov o = covariates_impl(on_grid, f, g, bo_row, a->ybo, bx_k, S->ybx[j], di,
                                       (float)b_k, m);
            k0 = fma(di * di, b2, k0);
            k1 = fma(di * 2, bd, k1);
            w  = fma(di, vb, w);
            bd = fma(di, b2, bd);
            b2 = fma(b_k, b_k, b2);
            vb = fma(y_k, b_k, vb);
            if (on_grid) {
                const double uw  = o.fy - w;
                const double den = (k0 + k1) - o.ff;
                const double sse = den > tol ? (uw * uw) / (den + tol) : 0;
                if (sse > S->hsse[j]) {
                    S->hsse[j] = sse;
                    S->hidx[j] = (int)i;
                }
            }
        }
    }
    for (size_t j = 0; j < p; ++j) {
        if (S->hidx[j] >= 0) {
            hinge_dsse[S->bcols[j]] = linear_dsse[S->bcols[j]] + S->hsse[j];
            hinge_cuts[S->bcols[j]] = a->X[(size_t)xcol * a->ldx + (size_t)k[S->hidx[j]]];
        }
    }
    return 0;
}

/*
 *  marslib.cc:41-148: evaluate every row of the (rows x m) row-major mask
 *  (row stride mask_stride) with an OpenMP loop over X columns. Outputs are
 *  (rows x m) row-major. threads <= 0 means min(64, processors).
 */
MO_EXPORT int mo_eval_all(void *h, double *lin, double *hin, double *cut, const bool *mask,
                          int rows, int mask_stride, int min_span, int end_span,
                          int linear_only, int threads, long *dgks_counter, char *err,
                          size_t errlen)
{
    mo_algo *a = (mo_algo *)h;
    if (min_span < 1) {
        set_err(err, errlen, "min_span must be >= 1");
        return -1;
    }
    int nprocs = 1;
#ifdef _OPENMP
    nprocs = omp_get_num_procs();
#endif
    threads = threads <= 0 ? (nprocs < 64 ? nprocs : 64) : (threads < nprocs ? threads : nprocs);
    if (threads > rows) {
        threads = rows;
    }
    if (threads < 1) {
        threads = 1;
    }
    const size_t m = a->m;
    int status = 0;
    long dgks = 0;
#pragma omp parallel num_threads(threads) reduction(+ : dgks)
    {
        mo_scratch S;
        scratch_alloc(&S, a->n, m);
        char local_err[160] = {0};
#pragma omp for schedule(static)
        for (int i = 0; i < rows; ++i) {
            int st;
#pragma omp atomic read
            st = status;
            if (st != 0) {
                continue;
            }
            int rc = eval_one(a, &S, lin + (size_t)i * m, hin + (size_t)i * m,
                              cut + (size_t)i * m, i, mask + (size_t)i * mask_stride,
                              min_span, end_span, linear_only != 0, &dgks, local_err,
                              sizeof(local_err));
            if (rc != 0) {
#pragma omp critical
                {
                    if (status == 0) {
                        status = rc;
                        set_err(err, errlen, local_err);
                    }
                }
            }
        }
        scratch_free(&S);
    }
    if (dgks_counter) {
        *dgks_counter += dgks;
    }
    return status;
}

/* marsalgo.cc:760-875. Returns the MSE, -1 if degenerate; *status -1 on error. */
MO_EXPORT double mo_append(void *h, char type, int xcol, int bcol, float hcut, int *status,
                           char *err, size_t errlen)
{
    mo_algo *a = (mo_algo *)h;
    *status = 0;
    if (a->m >= a->max_terms) {
        set_err(err, errlen, "basis matrix is full");
        *status = -1;
        return 0;
    }
    if (bcol < 0 || (size_t)bcol >= a->m) {
        char msg[80];
        snprintf(msg, sizeof(msg), "invalid basis column number: %d", bcol);
        set_err(err, errlen, msg);
        *status = -1;
        return 0;
    }
    if (xcol < 0 || (size_t)xcol >= a->p) {
        set_err(err, errlen, "invalid X column index");
        *status = -1;
        return 0;
    }
    if (type != 'l' && type != '+' && type != '-') {
        set_err(err, errlen, "invalid basis type");
        *status = -1;
        return 0;
    }
    const size_t n = a->n, m = a->m, ldBo = a->max_terms;
    const float  s  = a->s[xcol];
    const float *bp = a->B + (size_t)bcol * n;
    const float *xp = a->X + (size_t)xcol * a->ldx;
    float       *Bm = a->B + m * n;
    for (size_t i = 0; i < n; ++i) {
        float v;
        if (type == 'l') {
            v = s * bp[i] * xp[i];
        } else if (type == '+') {
            float t = xp[i] - hcut;
            v = s * bp[i] * ((t < 0.0f) ? 0.0f : t);   /* std::max(t, 0.0f) */
        } else {
            float t = hcut - xp[i];
            v = s * bp[i] * ((t < 0.0f) ? 0.0f : t);
        }
        Bm[i] = v;
    }
    double *v = (double *)malloc((n + 1) * sizeof(double));
    for (size_t i = 0; i < n; ++i) {
        v[i] = (double)Bm[i];
    }
    double raw2 = 0.0;
    for (size_t i = 0; i < n; ++i) {
        raw2 = fma(v[i], v[i], raw2);
    }
    const float raw = (float)sqrt(raw2);
    for (size_t i = 0; i < n; ++i) {
        Bm[i] /= raw;
    }
    const double w = mo_orthonormalize_col(n, m, v, a->Bo, ldBo, a->tol, NULL);
    double result = -1.0;
    if (w * w > a->tol) {
        for (size_t i = 0; i < n; ++i) {
            a->Bo[i * ldBo + m] = (float)v[i];
        }
        double ybo_m = 0.0;
        for (size_t i = 0; i < n; ++i) {
            ybo_m = fma((double)a->Bo[i * ldBo + m], (double)a->y[i], ybo_m);
        }
        /* marsalgo.cc:863-866. GCC's own contraction of this short loop is
         * unroll-dependent, so the reported MSE agrees with the reference to
         * a few ulp rather than bit for bit. */
        double ybo_sq = ybo_m * ybo_m;
        for (size_t j = 0; j < m; ++j) {
            ybo_sq = fma(a->ybo[j], a->ybo[j], ybo_sq);
        }
        const double mse = (1. - ybo_sq) / (double)n;
        if (mse >= -a->tol) {
            a->ybo[m] = ybo_m;
            a->m += 1;
            result = mse < 0.0 ? 0.0 : mse;
        }
    }
    free(v);
    return result;
}
