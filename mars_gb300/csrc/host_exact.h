// The fit state's set-up (marsalgo.cc:266-370) on the host, in the reference's
// exact operation order: the normalised weighted target, the intercept column,
// y . intercept, the target variance and the column scales of X. Everything
// after it -- evals and appends -- runs on the GPU.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace mgpu {

struct HostBasis {
    size_t n = 0, p = 0, ldx = 0;
    double tol = 0.0, yvar = 0.0;
    const float *X = nullptr;  // caller's X, column-major, column stride ldx (borrowed)
    std::vector<float> s;      // 1/rms per X column
    std::vector<float> y;      // normalised target
    std::vector<float> b0;     // the intercept column (normalised sqrt weights)
    double ybo0 = 0.0;         // y . b0

    // marsalgo.cc:266-370. Throws mgpu::Error with the reference's messages.
    void init(const float *X, const float *y, const float *w, size_t n, size_t p, size_t ldx);
};

// One candidate's exact values (marsalgo.cc:436-656 with kernels.cc:283-417):
// ybx of the orthonormalised column and the best hinge delta SSE with its row
// (-1 if none).
struct ExactResult {
    double ybx = 0.0;
    double hinge_sse = 0.0;
    int hinge_pos = -1;
    int hinge_row = -1;
};

// Cores this process may run on (its CPU affinity mask; at least 1).
int usable_cores();

}  // namespace mgpu
