// The exact append on the GPU: one new basis column in the reference's FP64
// order (marsalgo.cc:760-875, kernels.cc:194-281), every sequential chain of it
// evaluated exactly in parallel (xchain.cuh), one launch per chain.
#pragma once

#include "common.cuh"

#include <vector>

namespace mgpu {

// Device buffers of the append (one set per handle, bound to its stream).
struct XaBufs {
    DevBuf v0, v1;         // the f64 working column, two generations
    DevBuf rc, rs, rw, rb;  // chain records: chunks, sub-groups, warps, blocks
    DevBuf agg, g0, g1;    // next-chain aggregates per block; block entry guesses
    DevBuf res, ticket;    // chain results; the last-block ticket
    void bind(cudaStream_t st)
    {
        for (DevBuf *b : {&v0, &v1, &rc, &rs, &rw, &rb, &agg, &g0, &g1, &res, &ticket}) {
            b->bind(st);
        }
    }
};

// The fit state an append extends (device pointers; B and BoC column-major
// with column stride n).
struct XaFit {
    int n, m, max_terms;
    const float *X;
    size_t ldX;
    const float *s;  // column scales of X
    const float *y;  // the normalised weighted target
    float *B;
    float *BoC;
    double tol;
};

struct XaOutcome {
    double w2;      // squared norm of the projected column (its final pass)
    double ybo;     // y . the new orthonormal column, when w2 > tol
    bool stored;    // w2 > tol: column m of BoC holds the new orthonormal column
    bool dgks;      // the second Gram-Schmidt pass ran
};

// Builds column m of B from (type, xcol, bcol, h), orthonormalises it against
// columns 0..m-1 of BoC and, when its norm passes tol, stores it in column m of
// BoC and returns y . it. The caller accepts the column (the reference's MSE
// test, marsalgo.cc:863-870) and copies it to the row-major layouts.
XaOutcome append_exact(cudaStream_t st, const XaFit &fit, char type, int xcol, int bcol, float h,
                       XaBufs &bufs, long long *launches);

// kernels.cc:239-281 on a device column: v (n f64, device) orthonormalised
// against columns 0..m-1 of BoC (column-major, stride n) with the DGKS
// re-pass, and divided by its norm w when w^2 > tol. Returns w.
double orthonormalize_col_exact(cudaStream_t st, int n, int m, const float *BoC, double *v,
                                double tol, XaBufs &bufs, long long *launches, bool *dgks);

// T[j m + k] = sum_i BoC[i, k] * Bx[i, col(j)] (col null: j) for P candidates
// and m basis columns, every entry the reference's chain over the rows in order
// (kernels.cc:327-335) evaluated exactly in parallel, all entries side by side.
// Pays where the entries are few (a DGKS re-pass): the chains as written take
// n dependent FMA latencies whatever their number. Returns false (nothing
// launched) when there are more than 65535 entries.
bool tgemm_exact(cudaStream_t st, int n, int m, int P, const float *BoC, const float *Bx,
                 size_t ldBx, const int *col, double *T, XaBufs &bufs, long long *launches);

}  // namespace mgpu
