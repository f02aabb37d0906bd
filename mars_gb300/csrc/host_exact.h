// Host-side FP64 arithmetic in the reference's exact operation order.
//
// GB300's FP64 unit has a dependent-FMA latency of ~67 cycles (measured: 32 ns
// per step of a serial chain), while a Grace core runs the same chain at
// 0.66 ns per step. The reference's long serial reductions -- the modified
// Gram-Schmidt of append() and the per-candidate FP64 hinge sweep -- are
// therefore evaluated here on the host cores, bit for bit in the reference's
// order, for the few places that need exactly the reference's rounding: every
// append, and the candidates whose GPU scores lie within their error bound of
// a decision (the "contenders" of an epoch).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace mgpu {

struct HostBasis {
    size_t n = 0, p = 0, ldx = 0, max_terms = 0, m = 1;
    double tol = 0.0, yvar = 0.0;
    const float *X = nullptr;  // caller's X, column-major, column stride ldx (borrowed)
    std::vector<float> s;      // 1/rms per X column
    std::vector<float> y;      // normalised target
    std::vector<float> B;      // basis, column-major n x max_terms
    std::vector<float> BoC;    // orthonormal basis, column-major n x max_terms
    std::vector<float> BoR;    // orthonormal basis, row-major n x max_terms
    std::vector<double> ybo;   // Bo^T y per live column

    // marsalgo.cc:266-370. Throws mgpu::Error with the reference's messages.
    void init(const float *X, const float *y, const float *w, size_t n, size_t p, size_t ldx,
              size_t max_terms);
    // marsalgo.cc:760-875 (validation done by the caller). Returns the MSE or
    // -1; writes the new column m of B and Bo when accepted (and B[:, m] always).
    double append(char type, int xcol, int bcol, float h, long *dgks);
    double dsse() const;
};

// One candidate (input column xcol, parent basis column bcol) evaluated as the
// reference's eval() does for it (marsalgo.cc:436-656 with kernels.cc:283-417):
// ybx of the orthonormalised column, and, when perm is given (the stable
// descending order of X[:, xcol]), the best hinge delta SSE and its sorted
// position (-1 if none).
struct ExactResult {
    double ybx = 0.0;
    double hinge_sse = 0.0;
    int hinge_pos = -1;
    int hinge_row = -1;
    bool dgks = false;
};
ExactResult exact_candidate(const HostBasis &hb, int xcol, int bcol, const int32_t *perm,
                            int min_span, int head, int tail);

// Cores this process may run on (its CPU affinity mask; at least 1).
int usable_cores();

// Evaluate a list of candidates on up to `threads` host threads.
void exact_candidates(const HostBasis &hb, const std::vector<int> &xcol,
                      const std::vector<int> &bcol, const std::vector<const int32_t *> &perm,
                      int min_span, int head, int tail, std::vector<ExactResult> &out,
                      int threads);

}  // namespace mgpu
