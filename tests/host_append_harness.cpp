// The library's host-side basis (mars_gb300/csrc/host_exact.cpp) behind a few C
// entry points, so that the CPU tests can run its appends -- in order or over
// the host thread pool -- without a GPU.
#include "../mars_gb300/csrc/host_exact.h"

#include <cstring>
#include <string>

namespace mgpu {
void set_last_error(const std::string &) {}
}  // namespace mgpu

extern "C" {

void *ha_create(const float *X, const float *y, const float *w, size_t n, size_t p,
                size_t max_terms)
{
    auto *hb = new mgpu::HostBasis();
    hb->init(X, y, w, n, p, n, max_terms);
    return hb;
}

double ha_append(void *h, char type, int xcol, int bcol, float hinge, long *dgks)
{
    return static_cast<mgpu::HostBasis *>(h)->append(type, xcol, bcol, hinge, dgks);
}

size_t ha_nbasis(void *h) { return static_cast<mgpu::HostBasis *>(h)->m; }

// Column j of Bo (column-major copy) and of B, and ybo[j].
void ha_column(void *h, int j, float *bo, float *b)
{
    auto *hb = static_cast<mgpu::HostBasis *>(h);
    std::memcpy(bo, hb->BoC.data() + (size_t)j * hb->n, hb->n * sizeof(float));
    std::memcpy(b, hb->B.data() + (size_t)j * hb->n, hb->n * sizeof(float));
}

double ha_ybo(void *h, int j) { return static_cast<mgpu::HostBasis *>(h)->ybo[(size_t)j]; }

// Row i of the row-major copy of Bo.
void ha_bo_row(void *h, size_t i, float *out)
{
    auto *hb = static_cast<mgpu::HostBasis *>(h);
    std::memcpy(out, hb->BoR.data() + i * hb->max_terms, hb->max_terms * sizeof(float));
}

void ha_destroy(void *h) { delete static_cast<mgpu::HostBasis *>(h); }
}
