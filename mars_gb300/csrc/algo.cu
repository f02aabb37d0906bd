// Host side of the GB300 MARS forward pass: the fit state behind the C ABI
// (include/mars_gpu.h). One handle = the reference's MarsAlgo
// (marsalgo.cc:266-875) plus its device context (cuda/orthonormalize.cu),
// re-designed so that every candidate of an epoch is evaluated on the device
// in one call and the basis lives only in device memory.
#include "../../include/mars_gpu.h"
#include "common.cuh"
#include "fast.cuh"
#include "fp64.cuh"
#include "host_exact.h"
#include "tc.cuh"
#include "xappend.cuh"

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <limits>
#include <thread>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

using namespace mgpu;

namespace {
thread_local std::string g_last_error;

template <class F>
int guarded(F &&f)
{
    try {
        f();
        return MARS_GPU_OK;
    } catch (const Error &e) {
        g_last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc &) {
        g_last_error = "host allocation failed";
        return MARS_GPU_ENOMEM;
    } catch (const std::exception &e) {
        g_last_error = e.what();
        return MARS_GPU_ECUDA;
    }
}

}  // namespace

void mgpu::set_last_error(const std::string &msg) { g_last_error = msg; }

namespace {

double env_double(const char *name, double dflt)
{
    const char *v = std::getenv(name);
    return (v && *v) ? std::atof(v) : dflt;
}

enum Phase {
    PH_PROJECT,
    PH_DGKS,
    PH_NORMALIZE,
    PH_SWEEP,
    PH_SORT,
    PH_APPEND,
    PH_REDECIDE,
    PH_GATHER,
    PH_REDECIDE_GPU,
    PH_N
};

// Device time per phase, resolved after the stream is synchronised.
struct PhaseTimer {
    cudaStream_t st = nullptr;
    int redirect = -1;  // when >= 0, every phase is booked to this one
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> open;
    size_t used = 0;
    cudaEvent_t get()
    {
        if (used == pool.size()) {
            cudaEvent_t e;
            CUDA_CHECK(cudaEventCreate(&e));
            pool.push_back(e);
        }
        return pool[used++];
    }
    cudaEvent_t begin()
    {
        cudaEvent_t e = get();
        CUDA_CHECK(cudaEventRecord(e, st));
        return e;
    }
    void end(int phase, cudaEvent_t b)
    {
        cudaEvent_t e = get();
        CUDA_CHECK(cudaEventRecord(e, st));
        open.push_back({redirect >= 0 ? redirect : phase, {b, e}});
    }
    void resolve(double *ms)
    {
        for (auto &o : open) {
            float t = 0.f;
            if (cudaEventElapsedTime(&t, o.second.first, o.second.second) == cudaSuccess) {
                ms[o.first] += t;
            }
        }
        open.clear();
        used = 0;
    }
    ~PhaseTimer()
    {
        for (auto e : pool) {
            cudaEventDestroy(e);
        }
    }
};

// The streams, counters and scratch one FP64 evaluation runs on (the handle's).
struct Fp64Ctx {
    cudaStream_t st, st2, st3;
    cudaEvent_t ev_fork, ev_join, ev_s, ev_ybx;
    PhaseTimer *timer;
    mars_gpu_stats *stats;
    DevBuf *Bx, *T, *svec, *snew, *ybx, *hsse, *hrow, *fired, *nfired, *tasks, *stasks, *scal,
        *bsort, *bxsort, *cand, *part;
};

// Streams and events of one FP64 context: the main stream, the side stream of
// the hinge scalars and the one of the ybx chain, with their fork/join events.
struct Fp64Streams {
    cudaStream_t st = nullptr, st2 = nullptr, st3 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_s = nullptr, ev_ybx = nullptr;
    void create()
    {
        CUDA_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        CUDA_CHECK(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking));
        CUDA_CHECK(cudaStreamCreateWithFlags(&st3, cudaStreamNonBlocking));
        CUDA_CHECK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
        CUDA_CHECK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
        CUDA_CHECK(cudaEventCreateWithFlags(&ev_s, cudaEventDisableTiming));
        CUDA_CHECK(cudaEventCreateWithFlags(&ev_ybx, cudaEventDisableTiming));
    }
    ~Fp64Streams()
    {
        for (cudaStream_t x : {st, st2, st3}) {
            if (x) {
                cudaStreamSynchronize(x);
                cudaStreamDestroy(x);
            }
        }
        for (cudaEvent_t e : {ev_fork, ev_join, ev_s, ev_ybx}) {
            if (e) {
                cudaEventDestroy(e);
            }
        }
    }
};

}  // namespace

struct mars_gpu_algo {
    size_t n = 0, p = 0, max_terms = 0, ldbo = 0, m = 1;
    double tol = 0, yvar = 0;
    int precision = MARS_GPU_PREC_FP64;
    std::vector<double> ybo;
    // The handle's stream (st), with side streams for the hinge-sweep scalar
    // recurrences, which run concurrently with the projection, and for the
    // ybx chain, which runs concurrently with the sweep (fork/join events).
    Fp64Streams ss;
    cudaStream_t st = nullptr;
    PhaseTimer timer;
    double phase_ms[PH_N] = {0};
    cudaEvent_t span_begin = nullptr, span_end = nullptr;
    bool span_started = false;
    mars_gpu_stats stats;

    // Host copy of the basis, kept in the reference's exact arithmetic.
    HostBasis hb;
    XaBufs xa;  // the exact append's buffers
    // Resident state.
    DevBuf X, s, y, B, Bo, BoF, BoC, ybo_d, perm, xsort, ysort;
    std::vector<char> sorted;
    // Per-eval scratch (grow-only).
    DevBuf Bx, T, svec, snew, ybx, hsse, hrow, cand, fired, nfired, out, tasks, stasks, scal, part;
    DevBuf bsort, bxsort;  // per candidate: parent and normalised column in sorted order
    DevBuf fTp, fT, fmom, hflag;  // fast pass: split-K partials, T, parent moments, sweep flags
    // Fast pass on the tensor cores: split (hi, lo) copies of the basis, the
    // split coefficients and the kernels' error word; tc_cols basis columns
    // copied so far.
    DevBuf tcHiC, tcLoC, tcHiR, tcLoR, tcThi, tcTlo, tcErr, tcTab;
    size_t tc_cols = 0;
    // Fast pass: the basis row-major (BR, ldbr; br_cols columns copied), the
    // norms' partial sums, and the column-major candidates of the FP32 SIMT
    // projection before they are laid out by rows.
    DevBuf BR, fNpart, fBxc;
    size_t ldbr = 0, br_cols = 0;
    DevBuf sort_keys, sort_vals, sort_tmp;
    // Mixed mode: steps left to run on the exact path directly, after a step
    // that re-decided most of its candidates anyway.
    int mixed_skip = 0;

    Fp64Ctx ctx()
    {
        return {ss.st,  ss.st2, ss.st3, ss.ev_fork, ss.ev_join, ss.ev_s, ss.ev_ybx,
                &timer, &stats, &Bx,    &T,         &svec,      &snew,   &ybx,
                &hsse,  &hrow,  &fired, &nfired,    &tasks,     &stasks, &scal,
                &bsort, &bxsort, &cand, &part};
    }

    ~mars_gpu_algo()
    {
        if (span_begin) {
            cudaEventDestroy(span_begin);
        }
        if (span_end) {
            cudaEventDestroy(span_end);
        }
    }
};

namespace {

void sync(mars_gpu_algo *a) { CUDA_CHECK(cudaStreamSynchronize(a->st)); }

// The device-time span of a fit: from the start of its first eval to the end
// of its latest eval or append, on the handle's stream.
void span_mark_begin(mars_gpu_algo *a)
{
    if (!a->span_started) {
        CUDA_CHECK(cudaEventRecord(a->span_begin, a->st));
        a->span_started = true;
    }
}

void span_mark_end(mars_gpu_algo *a)
{
    if (a->span_started) {
        CUDA_CHECK(cudaEventRecord(a->span_end, a->st));
    }
}


// Column c of the row-major basis copies (f64, exact widening, and f32) from the f32 column.
__global__ void k_col_to_rows(const float *__restrict__ col, int n, double *__restrict__ Bo,
                              float *__restrict__ BoF, size_t ldbo, int c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        Bo[(size_t)i * ldbo + c] = (double)col[i];
        BoF[(size_t)i * ldbo + c] = col[i];
    }
}

void create_impl(mars_gpu_algo *a, const float *X, const float *y, const float *w, size_t n,
                 size_t p, size_t ldx, size_t max_terms)
{
    verify(ldx >= n || p <= 1, "X column stride smaller than the row count");
    verify(p <= 65535, "more than 65535 X columns");
    verify(n < (size_t)INT32_MAX, "more rows than the GPU path supports (2^31 - 1)");
    // The weighted, normalised target, the intercept and the column scales in
    // the reference's arithmetic (marsalgo.cc:266-370), on the host.
    verify(max_terms >= 1, "max_terms must be >= 1");
    a->hb.init(X, y, w, n, p, ldx);
    a->n = n;
    a->p = p;
    a->max_terms = max_terms;
    a->ldbo = round_up(max_terms, 4);
    a->m = 1;
    a->tol = a->hb.tol;
    a->yvar = a->hb.yvar;
    a->ybo.assign(1, a->hb.ybo0);
    std::memset(&a->stats, 0, sizeof(a->stats));
    a->ss.create();
    a->st = a->ss.st;
    for (DevBuf *b : {&a->X, &a->s, &a->y, &a->B, &a->Bo, &a->BoF, &a->BoC, &a->ybo_d, &a->perm,
                      &a->xsort, &a->ysort, &a->Bx, &a->T, &a->svec, &a->snew, &a->ybx,
                      &a->hsse, &a->hrow, &a->cand, &a->fired, &a->nfired, &a->out, &a->tasks,
                      &a->stasks, &a->scal, &a->part, &a->bsort, &a->bxsort, &a->fTp, &a->fT,
                      &a->fmom, &a->hflag, &a->sort_keys, &a->sort_vals, &a->sort_tmp,
                      &a->tcHiC, &a->tcLoC, &a->tcHiR, &a->tcLoR, &a->tcThi, &a->tcTlo,
                      &a->tcErr, &a->tcTab, &a->BR, &a->fNpart, &a->fBxc}) {
        b->bind(a->st);
    }
    a->xa.bind(a->st);
    CUDA_CHECK(cudaEventCreate(&a->span_begin));
    CUDA_CHECK(cudaEventCreate(&a->span_end));
    a->timer.st = a->st;

    // Device-resident state.
    a->stats.h2d_bytes += (long long)(sizeof(float) * (n * p + 3 * n + p));
    a->X.ensure(sizeof(float) * std::max<size_t>(1, n * p));
    if (n > 0 && p > 0) {
        CUDA_CHECK(cudaMemcpy2DAsync(a->X.ptr, n * sizeof(float), X, ldx * sizeof(float),
                                     n * sizeof(float), p, cudaMemcpyHostToDevice, a->st));
    }
    a->s.ensure(sizeof(float) * std::max<size_t>(1, p));
    if (p) {
        CUDA_CHECK(cudaMemcpyAsync(a->s.ptr, a->hb.s.data(), sizeof(float) * p,
                                   cudaMemcpyHostToDevice, a->st));
    }
    a->y.ensure(sizeof(float) * n);
    CUDA_CHECK(cudaMemcpyAsync(a->y.ptr, a->hb.y.data(), sizeof(float) * n,
                               cudaMemcpyHostToDevice, a->st));
    a->B.ensure(sizeof(float) * n * max_terms);
    a->BoC.ensure(sizeof(float) * n * max_terms);
    a->Bo.ensure(sizeof(double) * n * a->ldbo);
    CUDA_CHECK(cudaMemsetAsync(a->Bo.ptr, 0, sizeof(double) * n * a->ldbo, a->st));
    a->BoF.ensure(sizeof(float) * n * a->ldbo);
    CUDA_CHECK(cudaMemsetAsync(a->BoF.ptr, 0, sizeof(float) * n * a->ldbo, a->st));
    CUDA_CHECK(cudaMemcpyAsync(a->B.ptr, a->hb.b0.data(), sizeof(float) * n,
                               cudaMemcpyHostToDevice, a->st));
    CUDA_CHECK(cudaMemcpyAsync(a->BoC.ptr, a->hb.b0.data(), sizeof(float) * n,
                               cudaMemcpyHostToDevice, a->st));
    k_col_to_rows<<<(unsigned)ceil_div(n, 256), 256, 0, a->st>>>(
        a->BoC.as<float>(), (int)n, a->Bo.as<double>(), a->BoF.as<float>(), a->ldbo, 0);
    LAUNCH_CHECK();
    a->ybo_d.ensure(sizeof(double) * max_terms);
    CUDA_CHECK(cudaMemcpyAsync(a->ybo_d.ptr, &a->ybo[0], sizeof(double), cudaMemcpyHostToDevice,
                               a->st));
    a->sorted.assign(p, 0);
    sync(a);
}

// Candidate blocks: contiguous ranges of the (xcol-major) candidate list that
// never split an input column, each at most `cap` candidates.
std::vector<std::pair<int, int>> block_candidates(const std::vector<int> &cx, size_t cap)
{
    std::vector<std::pair<int, int>> blocks;
    const int P = (int)cx.size();
    int b0 = 0;
    while (b0 < P) {
        int b1 = b0;
        while (b1 < P) {
            int e = b1;
            while (e < P && cx[e] == cx[b1]) {
                ++e;
            }
            if (b1 > b0 && (size_t)(e - b0) > cap) {
                break;
            }
            b1 = e;
        }
        blocks.push_back({b0, b1});
        b0 = b1;
    }
    return blocks;
}

void ensure_sorted(mars_gpu_algo *a, const std::vector<int> &cols)
{
    std::vector<int> todo;
    for (int c : cols) {
        if (!a->sorted[c]) {
            todo.push_back(c);
        }
    }
    if (todo.empty()) {
        return;
    }
    const size_t np = a->n * a->p;
    a->perm.ensure(sizeof(int) * np);
    a->xsort.ensure(sizeof(float) * np);
    a->ysort.ensure(sizeof(float) * np);
    cudaEvent_t t0 = a->timer.begin();
    sort_columns(a->st, a->X.as<float>(), a->n, a->s.as<float>(), a->y.as<float>(), (int)a->n,
                 todo.data(), (int)todo.size(), a->perm.as<int>(), a->xsort.as<float>(),
                 a->ysort.as<float>(), a->sort_keys, a->sort_vals, a->sort_tmp,
                 &a->stats.kernel_launches);
    a->timer.end(PH_SORT, t0);
    for (int c : todo) {
        a->sorted[c] = 1;
    }
}

// Bytes of per-step scratch one eval may use (MARS_GPU_BLOCK_GB, default 45 %
// of the device's memory). A step whose candidates do not fit runs as several
// blocks, and on the FP64 path every block pays the full latency of its serial
// chains again, so the default is large.
double block_budget()
{
    const char *v = std::getenv("MARS_GPU_BLOCK_GB");
    if (v && *v) {
        return std::atof(v) * 1e9;
    }
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return 32e9;
    }
    return 0.45 * (double)tot;
}

// The FP64 evaluation of candidates [0, Pc) (device arrays cx/cb) on the
// context c. Fills c's ybx, and hsse/hrow unless linear_only. count_work: add
// the algorithmic FLOPs, bytes and knot evaluations to c's counters (not for
// re-decisions, whose candidates the fast pass has counted).
void eval_block_fp64(mars_gpu_algo *a, Fp64Ctx &c, int Pc, const int *cx_d, const int *cb_d,
                     const std::vector<int> &cx_h, int c0, int min_span, int head, int tail,
                     bool linear_only, bool count_work = true)
{
    const int n = (int)a->n, m = (int)a->m;
    float *Bx = c.Bx->as<float>();
    ProjectScratch ws;
    ws.T = c.T->as<double>();
    double *s = c.svec->as<double>();

    if (count_work) {
        c.stats->project_flops += 4.0 * (double)n * (double)m * (double)Pc;
    }
    // The sweep's scalar recurrences need only the parents, y and the sorted
    // inputs: start them on the side stream, concurrent with the projection.
    if (!linear_only) {
        std::vector<SweepTask> stasks;
        for (int b = 0; b < Pc;) {
            int e = b;
            while (e < Pc && cx_h[c0 + e] == cx_h[c0 + b]) {
                ++e;
            }
            for (int t = b; t < e; t += 32) {
                stasks.push_back({cx_h[c0 + b], t, std::min(32, e - t)});
            }
            b = e;
        }
        c.stasks->ensure(sizeof(SweepTask) * stasks.size());
        CUDA_CHECK(cudaMemcpyAsync(c.stasks->ptr, stasks.data(),
                                   sizeof(SweepTask) * stasks.size(), cudaMemcpyHostToDevice,
                                   c.st));
        c.stats->h2d_bytes += (long long)(sizeof(SweepTask) * stasks.size());
        // The gather is a wide, short kernel: on the handle's stream, so it does
        // not crowd out the single-wave chain kernels that the scalars overlap.
        gather_parents(c.st, a->perm.as<int>(), a->B.as<float>(), a->n, cx_d, cb_d, n, tail, Pc,
                       c.bsort->as<float>(), &c.stats->kernel_launches);
        CUDA_CHECK(cudaEventRecord(c.ev_fork, c.st));
        CUDA_CHECK(cudaStreamWaitEvent(c.st2, c.ev_fork, 0));
        hinge_scalars(c.st2, c.stasks->as<SweepTask>(), (int)stasks.size(), Pc, a->xsort.as<float>(),
                      a->ysort.as<float>(), c.bsort->as<float>(), n, head, tail, min_span,
                      c.scal->as<double>(), &c.stats->kernel_launches);
        CUDA_CHECK(cudaEventRecord(c.ev_join, c.st2));
    }
    cudaEvent_t t0 = c.timer->begin();
    FillSrc src{a->B.as<float>(), a->n, a->X.as<float>(), a->n, a->s.as<float>(), cx_d, cb_d};
    project_fp64(c.st, src, a->Bo.as<double>(), a->ldbo, a->BoC.as<float>(), &a->xa, n, m, Pc,
                 nullptr, Bx, a->n, s, ws,
                 &c.stats->kernel_launches);
    c.timer->end(PH_PROJECT, t0);

    t0 = c.timer->begin();
    dgks_gate(c.st, ws.T, m, Pc, s, a->tol, c.fired->as<int>(), c.nfired->as<int>(),
              &c.stats->kernel_launches);
    int nf = 0;
    CUDA_CHECK(cudaMemcpyAsync(&nf, c.nfired->ptr, sizeof(int), cudaMemcpyDeviceToHost, c.st));
    CUDA_CHECK(cudaStreamSynchronize(c.st));
    if (nf > 0) {
        StoredSrc src2{Bx, a->n, c.fired->as<int>()};
        project_fp64(c.st, src2, a->Bo.as<double>(), a->ldbo, a->BoC.as<float>(), &a->xa, n, m,
                     nf, c.fired->as<int>(), Bx,
                     a->n, c.snew->as<double>(), ws, &c.stats->kernel_launches);
        scatter_s(c.st, c.fired->as<int>(), nf, c.snew->as<double>(), s,
                  &c.stats->kernel_launches);
        c.stats->dgks_fired += nf;
    }
    c.timer->end(PH_DGKS, t0);

    t0 = c.timer->begin();
    // Few candidates (latency-bound chains): the ybx chain on its own stream,
    // the sweep storing partial scores that sweep_score finishes once ybx is
    // known. Many: the partial scores would cost more HBM traffic than the
    // overlap saves, so ybx comes first and the sweep scores directly.
    const double part_bytes =
        32.0 * Pc * (linear_only ? 0.0 : (double)sweep_grid_rows(head, tail, min_span));
    const bool defer = !linear_only && part_bytes <= env_double("MARS_GPU_DEFER_BYTES", 1e9);
    if (!defer) {
        normalize_ybx(c.st, Bx, a->n, n, Pc, s, a->tol, a->y.as<float>(), false,
                      c.ybx->as<double>(), &c.stats->kernel_launches);
        if (!linear_only) {
            gather_candidates(c.st, a->perm.as<int>(), Bx, a->n, cx_d, s, a->tol, n, tail, Pc,
                              c.bxsort->as<float>(), &c.stats->kernel_launches);
        }
    } else {
        c.part->ensure(std::max<size_t>(8, (size_t)part_bytes));
        CUDA_CHECK(cudaEventRecord(c.ev_s, c.st));
        CUDA_CHECK(cudaStreamWaitEvent(c.st3, c.ev_s, 0));
        normalize_ybx(c.st3, Bx, a->n, n, Pc, s, a->tol, a->y.as<float>(), false,
                      c.ybx->as<double>(), &c.stats->kernel_launches);
        CUDA_CHECK(cudaEventRecord(c.ev_ybx, c.st3));
        gather_candidates(c.st, a->perm.as<int>(), Bx, a->n, cx_d, s, a->tol, n, tail, Pc,
                          c.bxsort->as<float>(), &c.stats->kernel_launches);
    }
    c.timer->end(PH_NORMALIZE, t0);

    if (linear_only) {
        return;
    }
    std::vector<SweepTask> tasks;
    const int warps = sweep_warps(m, Pc);
    for (int b = 0; b < Pc;) {
        int e = b;
        while (e < Pc && cx_h[c0 + e] == cx_h[c0 + b]) {
            ++e;
        }
        if (count_work) {
            c.stats->sweep_bytes += (double)tail * (12.0 + 4.0 * m + 8.0 * (e - b));
        }
        for (int t = b; t < e; t += warps) {
            tasks.push_back({cx_h[c0 + b], t, std::min(warps, e - t)});
        }
        b = e;
    }
    c.tasks->ensure(sizeof(SweepTask) * tasks.size());
    CUDA_CHECK(cudaMemcpyAsync(c.tasks->ptr, tasks.data(), sizeof(SweepTask) * tasks.size(),
                               cudaMemcpyHostToDevice, c.st));
    c.stats->h2d_bytes += (long long)(sizeof(SweepTask) * tasks.size());
    CUDA_CHECK(cudaStreamWaitEvent(c.st, c.ev_join, 0));
    t0 = c.timer->begin();
    sweep_fp64(c.st, c.tasks->as<SweepTask>(), (int)tasks.size(), a->perm.as<int>(),
               a->xsort.as<float>(), c.bsort->as<float>(), c.bxsort->as<float>(),
               a->Bo.as<double>(), a->ldbo, a->ybo_d.as<double>(), c.ybx->as<double>(),
               c.scal->as<double>(), n, m, head, tail, min_span, a->tol, c.hsse->as<double>(),
               c.hrow->as<int>(), warps, &c.stats->kernel_launches,
               defer ? c.part->as<double>() : nullptr, sweep_split(m, Pc));
    if (defer) {
        CUDA_CHECK(cudaStreamWaitEvent(c.st, c.ev_ybx, 0));
        sweep_score(c.st, c.part->as<double>(), Pc, cx_d, a->perm.as<int>(),
                    c.ybx->as<double>(), n, head, tail, min_span, a->tol, c.hsse->as<double>(),
                    c.hrow->as<int>(), &c.stats->kernel_launches);
    }
    c.timer->end(PH_SWEEP, t0);
    if (count_work) {
        c.stats->knot_evals += (long long)Pc * sweep_grid_rows(head, tail, min_span);
    }
}


// Whether the fast projection runs on the tensor cores (MARS_GPU_TC, default
// 1; 0 selects the FP32 SIMT kernels).
bool use_tc(size_t m)
{
    return m <= (size_t)TC_MAX_M && env_double("MARS_GPU_TC", 1.0) != 0.0;
}

__global__ void k_col_to_rowmajor(const float *__restrict__ col, int n, float *__restrict__ BR,
                                  size_t ld, int c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        BR[(size_t)i * ld + c] = col[i];
    }
}

// The row-major copy of the basis B read by the fast pass, allocated on first
// use and brought up to the live basis.
void br_sync(mars_gpu_algo *a)
{
    if (!a->BR.ptr) {
        a->ldbr = round_up(a->max_terms, 4);
        a->BR.ensure(sizeof(float) * a->n * a->ldbr);
        CUDA_CHECK(cudaMemsetAsync(a->BR.ptr, 0, a->BR.bytes, a->st));
        a->br_cols = 0;
    }
    for (; a->br_cols < a->m; ++a->br_cols) {
        k_col_to_rowmajor<<<(unsigned)ceil_div(a->n, 256), 256, 0, a->st>>>(
            a->B.as<float>() + a->br_cols * a->n, (int)a->n, a->BR.as<float>(), a->ldbr,
            (int)a->br_cols);
        LAUNCH_CHECK();
        a->stats.kernel_launches += 1;
    }
}

// The split basis copies of the tensor-core projection, allocated on first
// use (zero-filled: rows past n and columns past m are read as zeros) and
// brought up to the live basis.
TcBasis tc_basis(mars_gpu_algo *a)
{
    TcBasis tb;
    tb.ldn = tc_ldn(a->n);
    tb.ldk = tc_ldk(a->max_terms);
    if (!a->tcHiC.ptr) {
        a->tcHiC.ensure(sizeof(float) * tb.ldn * a->max_terms);
        a->tcLoC.ensure(sizeof(float) * tb.ldn * a->max_terms);
        a->tcHiR.ensure(sizeof(float) * a->n * tb.ldk);
        a->tcLoR.ensure(sizeof(float) * a->n * tb.ldk);
        a->tcErr.ensure(sizeof(int));
        for (DevBuf *b : {&a->tcHiC, &a->tcLoC, &a->tcHiR, &a->tcLoR, &a->tcErr}) {
            CUDA_CHECK(cudaMemsetAsync(b->ptr, 0, b->bytes, a->st));
        }
        a->tc_cols = 0;
    }
    tb.hiC = a->tcHiC.as<float>();
    tb.loC = a->tcLoC.as<float>();
    tb.hiR = a->tcHiR.as<float>();
    tb.loR = a->tcLoR.as<float>();
    for (; a->tc_cols < a->m; ++a->tc_cols) {
        tc_store_column(a->st, a->BoC.as<float>() + a->tc_cols * a->n, (int)a->n,
                        (int)a->tc_cols, tb, &a->stats.kernel_launches);
    }
    return tb;
}

// Mixed precision (MARS_GPU_PREC_MIXED). Every candidate is ranked by the
// FP32 / FP64-carry fast pass on the GPU; the best-ranked ones -- the top
// MARS_GPU_MIXED_TOPK (default 4) by linear and by hinge delta SSE, and any
// within MARS_GPU_MIXED_BAND (default 2%) of the best fast value -- and the
// numerically unreliable ones (below) are
// re-evaluated on the FP64 GPU path in the reference's exact FP64 order, and
// the decisions come from those exact values: the
// re-decided candidates carry their exact delta SSE and knot, every other one
// its fast value, held strictly below the best exact value so the first
// maximum (mars.py:342-343) is always an exactly evaluated candidate.
void eval_mixed(mars_gpu_algo *a, const std::vector<int> &cx, const std::vector<int> &cb,
                int rows, int min_span, int head, int tail, bool linear_only, double *lin,
                double *hin, double *cut)
{
    const int n = (int)a->n, m = (int)a->m, P = (int)cx.size();
    const size_t cnt = (size_t)rows * m;
    for (size_t e = 0; e < cnt; ++e) {
        lin[e] = 0.0;
        hin[e] = 0.0;
        cut[e] = std::numeric_limits<double>::quiet_NaN();
    }
    if (P == 0) {
        return;
    }
    const int ks = fast_ksplit(n);
    const double budget = block_budget();
    const double ngrid = linear_only ? 0.0 : (double)sweep_grid_rows(head, tail, min_span);
    (void)ngrid;
    const bool tc = use_tc(a->m);
    // the FP32 SIMT projection keeps a column-major copy of its candidates too
    const double per = (tc ? 4.0 : 8.0) * n + 4.0 * m * (ks + 1) + 64.0;
    size_t cap = (size_t)std::max(1.0, budget / per);
    cap = std::min<size_t>(cap, 262144);
    const auto blocks = block_candidates(cx, cap);
    size_t maxPc = 0;
    for (auto &b : blocks) {
        maxPc = std::max<size_t>(maxPc, b.second - b.first);
    }
    // candidates row-major (ld ldr, set per block), so that the sweep reads a
    // sorted row's values of a block's candidates together
    a->Bx.ensure(sizeof(float) * a->n * round_up(maxPc, 4));
    a->fNpart.ensure(fast_norm_part_bytes(a->n, maxPc));
    if (!tc) {
        a->fBxc.ensure(sizeof(float) * a->n * maxPc);
    }
    br_sync(a);
    a->svec.ensure(sizeof(double) * maxPc);
    a->ybx.ensure(sizeof(double) * maxPc);
    a->hsse.ensure(sizeof(double) * 2 * maxPc);  // two sweep directions
    a->hrow.ensure(sizeof(int) * 2 * maxPc);
    TcBasis tb;
    if (tc) {
        tb = tc_basis(a);
        a->tcThi.ensure(sizeof(float) * maxPc * tb.ldk);
        a->tcTlo.ensure(sizeof(float) * maxPc * tb.ldk);
        a->tcTab.ensure(tc_tab_bytes(maxPc));
        size_t tp = 0;  // split-K partials of the largest block (the split count varies)
        for (auto &b : blocks) {
            const int Pc = b.second - b.first;
            tp = std::max(tp, (size_t)tc_ksplit(n, Pc) * (size_t)Pc);
        }
        a->fTp.ensure(sizeof(float) * tp * m);
    } else {
        a->fTp.ensure(sizeof(float) * (size_t)ks * maxPc * m);
    }
    a->fT.ensure(sizeof(float) * maxPc * m);
    a->fmom.ensure(sizeof(double) * 3 * maxPc);
    a->hflag.ensure(sizeof(int) * 2 * maxPc);
    a->cand.ensure(sizeof(int) * 2 * (size_t)P);
    int *cx_all = a->cand.as<int>(), *cb_all = cx_all + P;
    CUDA_CHECK(cudaMemcpyAsync(cx_all, cx.data(), sizeof(int) * P, cudaMemcpyHostToDevice, a->st));
    CUDA_CHECK(cudaMemcpyAsync(cb_all, cb.data(), sizeof(int) * P, cudaMemcpyHostToDevice, a->st));
    a->stats.h2d_bytes += (long long)(sizeof(int) * 2 * (size_t)P);

    // MARS_GPU_MIXED_RANK_ONLY=1: return the fast values as they are, with no
    // exact re-decision (to measure the fast pass's accuracy; not the
    // reference's decisions).
    const bool rank_only = env_double("MARS_GPU_MIXED_RANK_ONLY", 0.0) != 0.0;

    std::vector<double> fybx(P), fh(P, 0.0), fh2(2 * (size_t)P, 0.0), fs(P), fmom(3 * (size_t)P);
    std::vector<int> frow(P, -1), frow2(2 * (size_t)P, -1), fflag(2 * (size_t)P, 0);
    for (auto &b : blocks) {
        const int c0 = b.first, Pc = b.second - b.first;
        const int *cx_d = cx_all + c0, *cb_d = cb_all + c0;
        a->stats.project_flops += 4.0 * (double)n * (double)m * (double)Pc;
        cudaEvent_t t0 = a->timer.begin();
        FillSrc src{a->B.as<float>(), a->n, a->X.as<float>(), a->n, a->s.as<float>(), cx_d, cb_d};
        const size_t ldr = round_up((size_t)Pc, 4);
        if (tc) {
            const RowFillSrc rsrc{a->BR.as<float>(), a->ldbr, a->X.as<float>(), a->n,
                                  a->s.as<float>(), cx_d, cb_d};
            const TcScratch ws{a->fTp.as<float>(), a->fT.as<float>(), a->tcThi.as<float>(),
                               a->tcTlo.as<float>(), a->Bx.as<float>(), ldr,
                               a->svec.as<double>(), a->ybx.as<double>(), a->fmom.as<double>(),
                               a->tcErr.as<int>(), a->tcTab.ptr, a->fNpart.as<double>()};
            fast_project_tc(a->st, src, rsrc, tb, n, m, Pc, a->y.as<float>(), a->tol, ws,
                            &a->stats.kernel_launches);
        } else {
            FastScratch ws{a->fTp.as<float>(), a->fT.as<float>(), a->fBxc.as<float>(),
                           a->svec.as<double>(), a->ybx.as<double>(), a->fmom.as<double>()};
            fast_project(a->st, src, a->BoC.as<float>(), n, m, Pc, a->y.as<float>(), a->tol, ws,
                         &a->stats.kernel_launches);
            fast_to_rows(a->st, a->fBxc.as<float>(), n, Pc, a->Bx.as<float>(), ldr,
                         &a->stats.kernel_launches);
        }
        a->timer.end(PH_PROJECT, t0);
        if (!linear_only) {
            t0 = a->timer.begin();
            std::vector<FastTaskRec> tasks;
            std::vector<int> groups;
            for (int q = 0; q < Pc;) {
                int e = q;
                while (e < Pc && cx[c0 + e] == cx[c0 + q]) {
                    ++e;
                }
                groups.push_back(e - q);
                q = e;
            }
            const int warps = fast_sweep_warps(m, groups);
            for (int q = 0; q < Pc;) {
                int e = q;
                while (e < Pc && cx[c0 + e] == cx[c0 + q]) {
                    ++e;
                }
                a->stats.sweep_bytes += (double)n * (12.0 + 4.0 * m + 8.0 * (e - q));
                for (int t = q; t < e; t += warps) {
                    for (int dir = 0; dir < 2; ++dir) {
                        tasks.push_back({cx[c0 + q], t, std::min(warps, e - t), dir});
                    }
                }
                q = e;
            }
            a->tasks.ensure(sizeof(FastTaskRec) * tasks.size());
            CUDA_CHECK(cudaMemcpyAsync(a->tasks.ptr, tasks.data(),
                                       sizeof(FastTaskRec) * tasks.size(), cudaMemcpyHostToDevice,
                                       a->st));
            a->stats.h2d_bytes += (long long)(sizeof(FastTaskRec) * tasks.size());
            const FastSweepCols cols{a->BR.as<float>(), a->ldbr, cb_d,
                                     a->Bx.as<float>(), ldr,     a->svec.as<double>()};
            fast_sweep(a->st, a->tasks.as<FastTaskRec>(), (int)tasks.size(), a->perm.as<int>(),
                       a->xsort.as<float>(), a->ysort.as<float>(), cols, a->BoF.as<float>(), a->ldbo,
                       a->ybo_d.as<double>(), a->ybx.as<double>(), a->fmom.as<double>(), n, m,
                       head, tail, min_span, a->tol, env_double("MARS_GPU_MIXED_CUT_REL", 1e-7),
                       a->hsse.as<double>(), a->hrow.as<int>(), a->hflag.as<int>(), warps,
                       &a->stats.kernel_launches);
            a->timer.end(PH_SWEEP, t0);
            a->stats.knot_evals += (long long)Pc * sweep_grid_rows(head, tail, min_span);
            CUDA_CHECK(cudaMemcpyAsync(fh2.data() + 2 * (size_t)c0, a->hsse.ptr,
                                       sizeof(double) * 2 * Pc, cudaMemcpyDeviceToHost, a->st));
            CUDA_CHECK(cudaMemcpyAsync(frow2.data() + 2 * (size_t)c0, a->hrow.ptr,
                                       sizeof(int) * 2 * Pc, cudaMemcpyDeviceToHost, a->st));
            CUDA_CHECK(cudaMemcpyAsync(fflag.data() + 2 * (size_t)c0, a->hflag.ptr,
                                       sizeof(int) * 2 * Pc, cudaMemcpyDeviceToHost, a->st));
        }
        CUDA_CHECK(cudaMemcpyAsync(fybx.data() + c0, a->ybx.ptr, sizeof(double) * Pc,
                                   cudaMemcpyDeviceToHost, a->st));
        CUDA_CHECK(cudaMemcpyAsync(fs.data() + c0, a->svec.ptr, sizeof(double) * Pc,
                                   cudaMemcpyDeviceToHost, a->st));
        CUDA_CHECK(cudaMemcpyAsync(fmom.data() + 3 * (size_t)c0, a->fmom.ptr,
                                   sizeof(double) * 3 * Pc, cudaMemcpyDeviceToHost, a->st));
        a->stats.d2h_bytes += (long long)((linear_only ? 40 : 72) * (size_t)Pc);
        sync(a);
    }
    for (int j = 0; j < P && !linear_only; ++j) {  // the better of the two halves
        const double f0 = frow2[2 * (size_t)j] >= 0 ? fh2[2 * (size_t)j] : -1.0;
        const double f1 = frow2[2 * (size_t)j + 1] >= 0 ? fh2[2 * (size_t)j + 1] : -1.0;
        const int d = f1 > f0 ? 1 : 0;
        fh[j] = fh2[2 * (size_t)j + d];
        frow[j] = frow2[2 * (size_t)j + d];
    }

    if (rank_only) {
        // cut: the fast knot, or NaN where the candidate carries a flag
        const float *Xh = a->hb.X;
        const double degen = env_double("MARS_GPU_MIXED_DEGEN_REL", 1e-6);
        for (int j = 0; j < P; ++j) {
            const size_t idx = (size_t)cx[j] * m + cb[j];
            lin[idx] = fybx[j] * fybx[j];
            if (!linear_only && frow[j] >= 0) {
                hin[idx] = lin[idx] + fh[j];
                cut[idx] = (double)Xh[(size_t)frow[j] + (size_t)cx[j] * a->hb.ldx];
            }
            if (!linear_only && (fs[j] < degen * fmom[3 * (size_t)j + 2] ||
                                 fflag[2 * (size_t)j] || fflag[2 * (size_t)j + 1])) {
                cut[idx] = std::numeric_limits<double>::quiet_NaN();
            }
        }
        return;
    }

    // contenders: top-K and the band, by the fast linear and hinge values
    const auto t_host = std::chrono::steady_clock::now();
    const int topk = std::max(1, (int)env_double("MARS_GPU_MIXED_TOPK", 4));
    const double band = env_double("MARS_GPU_MIXED_BAND", 0.02);
    std::vector<double> flin(P), fhin(P, 0.0);
    for (int j = 0; j < P; ++j) {
        flin[j] = fybx[j] * fybx[j];
        if (!linear_only && frow[j] >= 0) {
            fhin[j] = flin[j] + fh[j];
        }
    }
    std::vector<char> contend(P, 0);
    auto pick = [&](const std::vector<double> &v) {
        std::vector<int> idx(P);
        for (int j = 0; j < P; ++j) {
            idx[j] = j;
        }
        const int k = std::min(topk, P);
        std::partial_sort(idx.begin(), idx.begin() + k, idx.end(),
                          [&](int x, int y) { return v[x] > v[y] || (v[x] == v[y] && x < y); });
        const double top = v[idx[0]];
        for (int q = 0; q < k; ++q) {
            contend[idx[q]] = 1;
        }
        for (int j = 0; j < P; ++j) {
            if (v[j] >= top * (1.0 - band)) {
                contend[j] = 1;
            }
        }
    };
    pick(flin);
    if (!linear_only) {
        pick(fhin);
        // Candidates whose reference evaluation is numerically unreliable --
        // a candidate column almost in the span (projected norm below
        // MARS_GPU_MIXED_DEGEN_REL, default 1e-6, of
        // its raw norm: every cut cancels), or a cut flagged by the sweep --
        // are re-decided too, since the reference's value there may be large.
        const double degen = env_double("MARS_GPU_MIXED_DEGEN_REL", 1e-6);
        for (int j = 0; j < P; ++j) {
            const bool dg = fs[j] < degen * fmom[3 * (size_t)j + 2];
            if (dg || fflag[2 * (size_t)j] || fflag[2 * (size_t)j + 1]) {
                contend[j] = 2;
                ++a->stats.redecided_flagged;
                a->stats.redecided_degenerate += dg ? 1 : 0;
            }
        }
    }
    // the exact re-decision of the contenders: the FP64 GPU path over them
    std::vector<int> ex_j, ex_x, ex_b;
    for (int j = 0; j < P; ++j) {
        if (contend[j]) {
            ex_j.push_back(j);
            ex_x.push_back(cx[j]);
            ex_b.push_back(cb[j]);
        }
    }
    std::vector<ExactResult> ex;
    if (!ex_j.empty()) {
        const int C = (int)ex_j.size();
        a->cand.ensure(sizeof(int) * 2 * (size_t)C);
        a->Bx.ensure(sizeof(float) * a->n * C);
        a->svec.ensure(sizeof(double) * C);
        a->ybx.ensure(sizeof(double) * C);
        a->hsse.ensure(sizeof(double) * C);
        a->hrow.ensure(sizeof(int) * C);
        if (!linear_only) {
            a->bsort.ensure(sizeof(float) * a->n * C);
            a->bxsort.ensure(sizeof(float) * a->n * C);
        }
        a->T.ensure(sizeof(double) * std::max<size_t>(1, (size_t)m * C));
        a->snew.ensure(sizeof(double) * C);
        a->fired.ensure(sizeof(int) * C);
        a->nfired.ensure(sizeof(int) * 4);
        if (!linear_only) {
            a->scal.ensure(sizeof(double) * 3 *
                           std::max<size_t>(1, (size_t)C * sweep_grid_rows(head, tail, min_span)));
        }
        int *ecx = a->cand.as<int>(), *ecb = ecx + C;
        CUDA_CHECK(cudaMemcpyAsync(ecx, ex_x.data(), sizeof(int) * C, cudaMemcpyHostToDevice,
                                   a->st));
        CUDA_CHECK(cudaMemcpyAsync(ecb, ex_b.data(), sizeof(int) * C, cudaMemcpyHostToDevice,
                                   a->st));
        a->stats.h2d_bytes += (long long)(sizeof(int) * 2 * (size_t)C);
        struct Redirect {
            PhaseTimer &t;
            ~Redirect() { t.redirect = -1; }
        } guard{a->timer};
        a->timer.redirect = PH_REDECIDE_GPU;
        Fp64Ctx c = a->ctx();
        eval_block_fp64(a, c, C, ecx, ecb, ex_x, 0, min_span, head, tail, linear_only, false);
        std::vector<double> eybx(C), ehs(C, 0.0);
        std::vector<int> ehr(C, -1);
        CUDA_CHECK(cudaMemcpyAsync(eybx.data(), a->ybx.ptr, sizeof(double) * C,
                                   cudaMemcpyDeviceToHost, a->st));
        if (!linear_only) {
            CUDA_CHECK(cudaMemcpyAsync(ehs.data(), a->hsse.ptr, sizeof(double) * C,
                                       cudaMemcpyDeviceToHost, a->st));
            CUDA_CHECK(cudaMemcpyAsync(ehr.data(), a->hrow.ptr, sizeof(int) * C,
                                       cudaMemcpyDeviceToHost, a->st));
        }
        a->stats.d2h_bytes += (long long)(20 * (size_t)C);
        sync(a);
        ex.resize(C);
        for (int q = 0; q < C; ++q) {
            ex[q].ybx = eybx[q];
            ex[q].hinge_sse = ehs[q];
            ex[q].hinge_row = ehr[q];
            ex[q].hinge_pos = ehr[q] >= 0 ? 0 : -1;
        }
    }
    a->stats.redecided += (long long)ex_j.size();

    // assemble: exact values for the contenders, fast values held below them for the rest
    double lbest = -std::numeric_limits<double>::infinity(), hbest = lbest;
    std::vector<double> elin(ex.size()), ehin(ex.size(), 0.0);
    for (size_t q = 0; q < ex.size(); ++q) {
        elin[q] = ex[q].ybx * ex[q].ybx;
        if (!linear_only && ex[q].hinge_pos >= 0) {
            ehin[q] = elin[q] + ex[q].hinge_sse;
        }
        lbest = std::max(lbest, elin[q]);
        hbest = std::max(hbest, ehin[q]);
    }
    const double lcap = std::nextafter(lbest, -std::numeric_limits<double>::infinity());
    const double hcap = std::nextafter(hbest, -std::numeric_limits<double>::infinity());
    const float *Xh = a->hb.X;
    for (int j = 0; j < P; ++j) {
        if (contend[j]) {
            continue;
        }
        const size_t idx = (size_t)cx[j] * m + cb[j];
        lin[idx] = std::min(flin[j], lcap);
        if (!linear_only && frow[j] >= 0) {
            hin[idx] = std::min(fhin[j], hcap);
            cut[idx] = (double)Xh[(size_t)frow[j] + (size_t)cx[j] * a->hb.ldx];
        }
    }
    for (size_t q = 0; q < ex.size(); ++q) {
        const int j = ex_j[q];
        const size_t idx = (size_t)cx[j] * m + cb[j];
        lin[idx] = elin[q];
        if (!linear_only && ex[q].hinge_pos >= 0) {
            hin[idx] = ehin[q];
            cut[idx] = (double)Xh[(size_t)ex[q].hinge_row + (size_t)cx[j] * a->hb.ldx];
        }
    }
    a->phase_ms[PH_REDECIDE] +=
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_host).count();
}

void eval_impl(mars_gpu_algo *a, const bool *mask, int rows, int mask_stride, int min_span,
               int end_span, int linear_only, double *sse0, double *lin, double *hin, double *cut)
{
    verify(rows >= 0 && (size_t)rows <= a->p, "invalid X column index");
    verify(min_span >= 1, "min_span must be >= 1");
    verify(end_span >= 0, "end_span must be >= 0");
    verify(rows == 0 || mask != nullptr, "mask is null");
    const int m = (int)a->m, n = (int)a->n;
    verify(mask_stride >= m || rows <= 1, "mask row stride smaller than nbasis");
    a->stats.evals += 1;
    span_mark_begin(a);

    std::vector<int> cx, cb, cols;
    for (int i = 0; i < rows; ++i) {
        bool any = false;
        for (int j = 0; j < m; ++j) {
            if (mask[(size_t)i * mask_stride + j]) {
                cx.push_back(i);
                cb.push_back(j);
                any = true;
            }
        }
        if (any) {
            cols.push_back(i);
        }
    }
    const int P = (int)cx.size();
    a->stats.candidates += P;
    // Mixed mode runs the fast pass unless a recent step re-decided more than
    // MARS_GPU_MIXED_FALLBACK (default half) of its candidates exactly: then
    // the next MARS_GPU_MIXED_FALLBACK_STEPS (7) steps take the exact path
    // directly (same decisions, no wasted fast pass), and the fast pass is
    // tried again.
    const bool use_fast = a->precision == MARS_GPU_PREC_MIXED && a->mixed_skip == 0;
    if (a->precision == MARS_GPU_PREC_MIXED && !use_fast) {
        --a->mixed_skip;
        a->stats.evals_exact += 1;
    }
    if (use_fast) {
        const int head = end_span;
        const int tail = head < n ? n - head : 0;
        if (P > 0 && !linear_only) {
            ensure_sorted(a, cols);
        }
        const long long before = a->stats.redecided;
        eval_mixed(a, cx, cb, rows, min_span, head, tail, linear_only != 0, lin, hin, cut);
        if (P > 0 && !linear_only &&
            (double)(a->stats.redecided - before) >
                env_double("MARS_GPU_MIXED_FALLBACK", 0.5) * (double)P) {
            a->mixed_skip = (int)env_double("MARS_GPU_MIXED_FALLBACK_STEPS", 7.0);
        }
        span_mark_end(a);
        sync(a);
        a->timer.resolve(a->phase_ms);
        if (sse0) {
            double s = 0.0;
            for (double v : a->ybo) {
                s = std::fma(v, v, s);
            }
            *sse0 = s;
        }
        return;
    }
    const size_t cnt = (size_t)rows * m;
    a->out.ensure(sizeof(double) * 3 * std::max<size_t>(cnt, 1));
    double *o_lin = a->out.as<double>(), *o_hin = o_lin + cnt, *o_cut = o_hin + cnt;
    fill_outputs(a->st, rows, m, o_lin, o_hin, o_cut, &a->stats.kernel_launches);

    const int head = end_span;
    const int tail = head < n ? n - head : 0;
    if (P > 0) {
        if (!linear_only) {
            ensure_sorted(a, cols);
        }
        const double budget = block_budget();
        // Candidate columns per block: the Bx scratch budget, and at most
        // 2^18 so every per-column grid dimension stays within 65535 blocks.
        const double ngrid = linear_only ? 0.0 : (double)sweep_grid_rows(head, tail, min_span);
        const double sorted_b = linear_only ? 0.0 : 8.0 * n;  // bsort + bxsort
        size_t cap = (size_t)std::max(
            1.0, budget / (4.0 * n + sorted_b + 24.0 * ngrid + 64.0 * m + 64.0));
        cap = std::min<size_t>(cap, 262144);
        const auto blocks = block_candidates(cx, cap);
        size_t maxPc = 0;
        for (auto &b : blocks) {
            maxPc = std::max<size_t>(maxPc, b.second - b.first);
        }
        a->Bx.ensure(sizeof(float) * a->n * maxPc);
        a->T.ensure(sizeof(double) * std::max<size_t>(1, (size_t)m * maxPc));
        a->svec.ensure(sizeof(double) * maxPc);
        a->snew.ensure(sizeof(double) * maxPc);
        a->ybx.ensure(sizeof(double) * maxPc);
        a->hsse.ensure(sizeof(double) * maxPc);
        a->hrow.ensure(sizeof(int) * maxPc);
        if (!linear_only) {
            a->scal.ensure(sizeof(double) * 3 *
                           std::max<size_t>(1, maxPc * (size_t)sweep_grid_rows(head, tail, min_span)));
            a->bsort.ensure(sizeof(float) * a->n * maxPc);
            a->bxsort.ensure(sizeof(float) * a->n * maxPc);
        }
        a->fired.ensure(sizeof(int) * maxPc);
        a->nfired.ensure(sizeof(int) * 4);
        a->cand.ensure(sizeof(int) * 2 * (size_t)P);
        a->stats.h2d_bytes += (long long)(sizeof(int) * 2 * (size_t)P);
        int *cx_all = a->cand.as<int>(), *cb_all = cx_all + P;
        CUDA_CHECK(cudaMemcpyAsync(cx_all, cx.data(), sizeof(int) * P, cudaMemcpyHostToDevice,
                                   a->st));
        CUDA_CHECK(cudaMemcpyAsync(cb_all, cb.data(), sizeof(int) * P, cudaMemcpyHostToDevice,
                                   a->st));
        for (auto &b : blocks) {
            const int c0 = b.first, Pc = b.second - b.first;
            const int *cx_d = cx_all + c0, *cb_d = cb_all + c0;
            Fp64Ctx c = a->ctx();
            eval_block_fp64(a, c, Pc, cx_d, cb_d, cx, c0, min_span, head, tail,
                            linear_only != 0);
            assemble_outputs(a->st, Pc, cx_d, cb_d, m, a->ybx.as<double>(), a->hsse.as<double>(),
                             a->hrow.as<int>(), a->X.as<float>(), a->n, linear_only != 0, o_lin,
                             o_hin, o_cut, &a->stats.kernel_launches);
        }
    }
    if (cnt) {
        CUDA_CHECK(cudaMemcpyAsync(lin, o_lin, sizeof(double) * cnt, cudaMemcpyDeviceToHost, a->st));
        CUDA_CHECK(cudaMemcpyAsync(hin, o_hin, sizeof(double) * cnt, cudaMemcpyDeviceToHost, a->st));
        CUDA_CHECK(cudaMemcpyAsync(cut, o_cut, sizeof(double) * cnt, cudaMemcpyDeviceToHost, a->st));
    }
    a->stats.d2h_bytes += (long long)(3 * sizeof(double) * cnt);
    span_mark_end(a);
    sync(a);
    a->timer.resolve(a->phase_ms);
    if (sse0) {
        double s = 0.0;
        for (double v : a->ybo) {
            s = std::fma(v, v, s);
        }
        *sse0 = s;
    }
}

double append_impl(mars_gpu_algo *a, char type, int xcol, int bcol, float h)
{
    verify(a->m < a->max_terms, "basis matrix is full", MARS_GPU_EFULL);
    if (bcol < 0 || (size_t)bcol >= a->m) {
        char msg[80];
        std::snprintf(msg, sizeof(msg), "invalid basis column number: %d", bcol);
        throw Error(MARS_GPU_EINVAL, msg);
    }
    verify(xcol >= 0 && (size_t)xcol < a->p, "invalid X column index");
    verify(type == 'l' || type == '+' || type == '-', "invalid basis type");
    const size_t n = a->n, m = a->m;
    // The reference's Gram-Schmidt in its FP64 order, every chain exact and
    // parallel on the GPU (xappend.cuh); the MSE test on the host.
    cudaEvent_t t0 = a->timer.begin();
    const XaFit fit{(int)n, (int)m, (int)a->max_terms, a->X.as<float>(), n, a->s.as<float>(),
                    a->y.as<float>(), a->B.as<float>(), a->BoC.as<float>(), a->tol};
    const XaOutcome o = append_exact(a->st, fit, type, xcol, bcol, h, a->xa,
                                     &a->stats.kernel_launches);
    a->stats.dgks_fired += o.dgks ? 1 : 0;
    a->stats.d2h_bytes += (long long)(sizeof(double) * (m + 4));
    double mse = -1.0;
    if (o.stored) {
        // marsalgo.cc:859-870
        double ybo_sq = o.ybo * o.ybo;
        for (double e : a->ybo) {
            ybo_sq = std::fma(e, e, ybo_sq);
        }
        const double r = (1. - ybo_sq) / (double)n;
        if (r >= -a->tol) {
            k_col_to_rows<<<(unsigned)ceil_div(n, 256), 256, 0, a->st>>>(
                a->BoC.as<float>() + m * n, (int)n, a->Bo.as<double>(), a->BoF.as<float>(),
                a->ldbo, (int)m);
            LAUNCH_CHECK();
            a->stats.kernel_launches += 1;
            CUDA_CHECK(cudaMemcpyAsync(a->ybo_d.as<double>() + m, &o.ybo, sizeof(double),
                                       cudaMemcpyHostToDevice, a->st));
            a->stats.h2d_bytes += (long long)sizeof(double);
            a->ybo.push_back(o.ybo);
            a->m = m + 1;
            mse = r < 0.0 ? 0.0 : r;
        }
    }
    a->timer.end(PH_APPEND, t0);
    span_mark_end(a);
    sync(a);
    a->timer.resolve(a->phase_ms);
    return mse;
}

// The Gram matrix Q^T Q and Q^T y of the live basis (FP64 chains over the
// rows), and from them, for each leading basis of k + 1 columns, max |Q^T Q - I|
// and 1 - sum(ybo^2). Stored columns never change after their append, so
// entry k is what the fit's step that made k + 1 columns would have measured.
void orth_error_by_terms(mars_gpu_algo *a, std::vector<double> &mx, std::vector<double> &rss)
{
    const int n = (int)a->n, m = (int)a->m;
    DevBuf T;
    T.ensure(sizeof(double) * (size_t)m * (m + 1));
    StoredSrc q{a->BoC.as<float>(), a->n, nullptr};
    tgemm_fp64(a->st, q, a->Bo.as<double>(), a->ldbo, n, m, m, T.as<double>(),
               &a->stats.kernel_launches);
    std::vector<double> G((size_t)m * m);
    CUDA_CHECK(cudaMemcpyAsync(G.data(), T.ptr, sizeof(double) * m * m, cudaMemcpyDeviceToHost,
                               a->st));
    StoredSrc yy{a->y.as<float>(), a->n, nullptr};
    tgemm_fp64(a->st, yy, a->Bo.as<double>(), a->ldbo, n, m, 1, T.as<double>(),
               &a->stats.kernel_launches);
    std::vector<double> r(m);
    CUDA_CHECK(cudaMemcpyAsync(r.data(), T.ptr, sizeof(double) * m, cudaMemcpyDeviceToHost,
                               a->st));
    sync(a);
    mx.assign(m, 0.0);
    rss.assign(m, 0.0);
    double run = 0.0, rs = 0.0;
    for (int k = 0; k < m; ++k) {
        // the new row and column k of the leading block
        for (int c = 0; c <= k; ++c) {
            const double d = std::fabs(G[(size_t)k * m + c] - (k == c ? 1.0 : 0.0));
            const double e = std::fabs(G[(size_t)c * m + k] - (k == c ? 1.0 : 0.0));
            run = std::max(run, std::max(d, e));
        }
        rs = std::fma(r[k], r[k], rs);
        mx[k] = run;
        rss[k] = 1.0 - rs;
    }
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *mars_gpu_last_error(void) { return g_last_error.c_str(); }

int mars_gpu_device_count(void)
{
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return c;
}

int mars_gpu_create(const float *X, const float *y, const float *w, size_t n, size_t p,
                    size_t ldx, size_t max_terms, mars_gpu_algo **out)
{
    if (!out) {
        g_last_error = "null output handle";
        return MARS_GPU_EINVAL;
    }
    *out = nullptr;
    mars_gpu_algo *a = nullptr;
    int rc = guarded([&] {
        verify(mars_gpu_device_count() > 0, "no CUDA device is visible", MARS_GPU_ECUDA);
        verify((X || n * p == 0) && y && w, "null input array");
        a = new mars_gpu_algo();
        create_impl(a, X, y, w, n, p, ldx, max_terms);
    });
    if (rc != MARS_GPU_OK) {
        delete a;
        return rc;
    }
    *out = a;
    return MARS_GPU_OK;
}

int mars_gpu_destroy(mars_gpu_algo *algo)
{
    delete algo;
    return MARS_GPU_OK;
}

int mars_gpu_nbasis(const mars_gpu_algo *a, int *out)
{
    if (!a || !out) {
        g_last_error = "null argument";
        return MARS_GPU_EINVAL;
    }
    *out = (int)a->m;
    return MARS_GPU_OK;
}

int mars_gpu_yvar(const mars_gpu_algo *a, double *out)
{
    if (!a || !out) {
        g_last_error = "null argument";
        return MARS_GPU_EINVAL;
    }
    *out = a->yvar;
    return MARS_GPU_OK;
}

int mars_gpu_dsse(const mars_gpu_algo *a, double *out)
{
    if (!a || !out) {
        g_last_error = "null argument";
        return MARS_GPU_EINVAL;
    }
    double s = 0.0;
    for (double v : a->ybo) {
        s = std::fma(v, v, s);
    }
    *out = s;
    return MARS_GPU_OK;
}

int mars_gpu_set_precision(mars_gpu_algo *a, int mode)
{
    return guarded([&] {
        verify(a != nullptr, "null handle");
        verify(mode == MARS_GPU_PREC_FP64 || mode == MARS_GPU_PREC_MIXED,
               "unknown precision mode");
        if (mode == MARS_GPU_PREC_MIXED && a->precision != mode) {
            a->sorted.assign(a->p, 0);  // re-sort so the host gets the permutations too
        }
        a->precision = mode;
        a->mixed_skip = 0;
    });
}

int mars_gpu_eval(mars_gpu_algo *a, const bool *mask, int rows, int mask_stride, int min_span,
                  int end_span, int linear_only, double *sse0, double *linear, double *hinge,
                  double *cut)
{
    return guarded([&] {
        verify(a != nullptr, "null handle");
        verify(rows == 0 || (linear && hinge && cut), "null output array");
        eval_impl(a, mask, rows, mask_stride, min_span, end_span, linear_only, sse0, linear, hinge,
                  cut);
    });
}

int mars_gpu_append(mars_gpu_algo *a, char type, int xcol, int bcol, float h, double *mse)
{
    return guarded([&] {
        verify(a != nullptr && mse != nullptr, "null argument");
        *mse = append_impl(a, type, xcol, bcol, h);
    });
}

int mars_gpu_get_stats(const mars_gpu_algo *a, mars_gpu_stats *out)
{
    if (!a || !out) {
        g_last_error = "null argument";
        return MARS_GPU_EINVAL;
    }
    *out = a->stats;
    out->ms_project = a->phase_ms[PH_PROJECT];
    out->ms_dgks = a->phase_ms[PH_DGKS];
    out->ms_normalize = a->phase_ms[PH_NORMALIZE];
    out->ms_sweep = a->phase_ms[PH_SWEEP];
    out->ms_sort = a->phase_ms[PH_SORT];
    out->ms_append = a->phase_ms[PH_APPEND];
    out->ms_redecide = a->phase_ms[PH_REDECIDE];
    out->ms_gather = a->phase_ms[PH_GATHER];
    out->ms_redecide_gpu = a->phase_ms[PH_REDECIDE_GPU];
    out->ms_span = 0.0;
    if (a->span_started) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, a->span_begin, a->span_end) == cudaSuccess) {
            out->ms_span = t;
        } else {
            cudaGetLastError();
        }
    }
    return MARS_GPU_OK;
}

int mars_gpu_pool_used_bytes(size_t *out)
{
    return guarded([&] {
        verify(out != nullptr, "null argument");
        verify(mars_gpu_device_count() > 0, "no CUDA device is visible", MARS_GPU_ECUDA);
        unsigned long long used = 0;  // the attribute is a 64-bit count
        CUDA_CHECK(cudaMemPoolGetAttribute(device_pool(), cudaMemPoolAttrUsedMemCurrent, &used));
        *out = (size_t)used;
    });
}

int mars_gpu_orth_error(mars_gpu_algo *a, double *max_abs, double *rss)
{
    return guarded([&] {
        verify(a != nullptr, "null handle");
        std::vector<double> mx, rs;
        orth_error_by_terms(a, mx, rs);
        if (max_abs) {
            *max_abs = mx.empty() ? 0.0 : mx.back();
        }
        if (rss) {
            *rss = rs.empty() ? 1.0 : rs.back();
        }
    });
}

int mars_gpu_orth_error_by_terms(mars_gpu_algo *a, double *max_abs, double *rss, size_t cap,
                                 size_t *count)
{
    return guarded([&] {
        verify(a != nullptr, "null handle");
        std::vector<double> mx, rs;
        orth_error_by_terms(a, mx, rs);
        const size_t k = std::min(cap, mx.size());
        for (size_t j = 0; j < k; ++j) {
            if (max_abs) {
                max_abs[j] = mx[j];
            }
            if (rss) {
                rss[j] = rs[j];
            }
        }
        if (count) {
            *count = mx.size();
        }
    });
}

int mars_gpu_orthonormalize(size_t n, size_t m, size_t p, const float *B, size_t ldB,
                            const float *x, const int *mask, const float *Bo, size_t ldBo,
                            float *Bx, size_t ldBx, double *s_out, double tol, long *dgks)
{
    return guarded([&] {
        verify(mars_gpu_device_count() > 0, "no CUDA device is visible", MARS_GPU_ECUDA);
        verify(n >= 1 && p >= 1, "empty problem");
        verify(ldB >= n && ldBx >= n && ldBo >= m, "leading dimension smaller than the data");
        verify(p <= 262144, "too many candidate columns for one call");
        int nbcols = 0;
        for (size_t j = 0; j < p; ++j) {
            verify(mask[j] >= 0, "negative basis index in mask");
            nbcols = std::max(nbcols, mask[j] + 1);
        }
        cudaStream_t st;
        CUDA_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        DevBuf dB, dx, dBo, dBx, dT, ds, dsn, dybx, dcand, dfired, dnf, dy, dsx;
        long long launches = 0;
        dB.ensure(sizeof(float) * n * nbcols);
        CUDA_CHECK(cudaMemcpy2DAsync(dB.ptr, n * sizeof(float), B, ldB * sizeof(float),
                                     n * sizeof(float), nbcols, cudaMemcpyHostToDevice, st));
        dx.ensure(sizeof(float) * n);
        CUDA_CHECK(cudaMemcpyAsync(dx.ptr, x, sizeof(float) * n, cudaMemcpyHostToDevice, st));
        const size_t ldbo = std::max<size_t>(ldBo, 1);
        dBo.ensure(sizeof(float) * n * ldbo);
        CUDA_CHECK(cudaMemcpyAsync(dBo.ptr, Bo, sizeof(float) * n * ldbo, cudaMemcpyHostToDevice, st));
        float one = 1.0f;
        dsx.ensure(sizeof(float));
        CUDA_CHECK(cudaMemcpyAsync(dsx.ptr, &one, sizeof(float), cudaMemcpyHostToDevice, st));
        dcand.ensure(sizeof(int) * 2 * p);
        std::vector<int> zeros(p, 0);
        CUDA_CHECK(cudaMemcpyAsync(dcand.ptr, zeros.data(), sizeof(int) * p, cudaMemcpyHostToDevice, st));
        CUDA_CHECK(cudaMemcpyAsync(dcand.as<int>() + p, mask, sizeof(int) * p,
                                   cudaMemcpyHostToDevice, st));
        dBx.ensure(sizeof(float) * n * p);
        dT.ensure(sizeof(double) * std::max<size_t>(1, m * p));
        ds.ensure(sizeof(double) * p);
        dsn.ensure(sizeof(double) * p);
        dybx.ensure(sizeof(double) * p);
        dfired.ensure(sizeof(int) * p);
        dnf.ensure(sizeof(int));
        dy.ensure(sizeof(float) * n);
        CUDA_CHECK(cudaMemsetAsync(dy.ptr, 0, sizeof(float) * n, st));
        ProjectScratch ws{dT.as<double>()};
        FillSrc src{dB.as<float>(), n, dx.as<float>(), n, dsx.as<float>(), dcand.as<int>(),
                    dcand.as<int>() + p};
        project_fp64(st, src, dBo.as<float>(), ldbo, nullptr, nullptr, (int)n, (int)m, (int)p,
                     nullptr,
                     dBx.as<float>(), n, ds.as<double>(), ws, &launches);
        dgks_gate(st, dT.as<double>(), (int)m, (int)p, ds.as<double>(), tol, dfired.as<int>(),
                  dnf.as<int>(), &launches);
        int nf = 0;
        CUDA_CHECK(cudaMemcpyAsync(&nf, dnf.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        if (nf > 0) {
            StoredSrc s2{dBx.as<float>(), n, dfired.as<int>()};
            project_fp64(st, s2, dBo.as<float>(), ldbo, nullptr, nullptr, (int)n, (int)m, nf,
                         dfired.as<int>(),
                         dBx.as<float>(), n, dsn.as<double>(), ws, &launches);
            scatter_s(st, dfired.as<int>(), nf, dsn.as<double>(), ds.as<double>(), &launches);
        }
        std::vector<double> sh(p);
        CUDA_CHECK(cudaMemcpyAsync(sh.data(), ds.ptr, sizeof(double) * p, cudaMemcpyDeviceToHost, st));
        normalize_ybx(st, dBx.as<float>(), n, (int)n, (int)p, ds.as<double>(), tol, dy.as<float>(),
                      true, dybx.as<double>(), &launches);
        CUDA_CHECK(cudaMemcpy2DAsync(Bx, ldBx * sizeof(float), dBx.ptr, n * sizeof(float),
                                     n * sizeof(float), p, cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        cudaStreamDestroy(st);
        if (s_out) {
            std::memcpy(s_out, sh.data(), sizeof(double) * p);
        }
        if (dgks) {
            *dgks += nf;
        }
    });
}

int mars_gpu_orthonormalize_col(size_t n, size_t m, double *v, const float *Bo, size_t ldBo,
                                double tol, double *w_out, long *dgks)
{
    return guarded([&] {
        verify(mars_gpu_device_count() > 0, "no CUDA device is visible", MARS_GPU_ECUDA);
        verify(n >= 1, "empty problem");
        cudaStream_t st;
        CUDA_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        std::vector<float> colmajor(n * std::max<size_t>(m, 1));
        for (size_t j = 0; j < m; ++j) {
            for (size_t i = 0; i < n; ++i) {
                colmajor[j * n + i] = Bo[i * ldBo + j];
            }
        }
        DevBuf dBoC, dv;
        long long launches = 0;
        dBoC.ensure(sizeof(float) * colmajor.size());
        CUDA_CHECK(cudaMemcpyAsync(dBoC.ptr, colmajor.data(), sizeof(float) * colmajor.size(),
                                   cudaMemcpyHostToDevice, st));
        dv.ensure(sizeof(double) * n);
        CUDA_CHECK(cudaMemcpyAsync(dv.ptr, v, sizeof(double) * n, cudaMemcpyHostToDevice, st));
        double w = 0.0;
        {
            XaBufs xa;
            bool fired = false;
            w = orthonormalize_col_exact(st, (int)n, (int)m, dBoC.as<float>(), dv.as<double>(),
                                         tol, xa, &launches, &fired);
            if (dgks && fired) {
                *dgks += 1;
            }
            CUDA_CHECK(cudaMemcpyAsync(v, dv.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
            CUDA_CHECK(cudaStreamSynchronize(st));
        }
        cudaStreamDestroy(st);
        if (w_out) {
            *w_out = w;
        }
    });
}

}  // extern "C"
