"""Seeded synthetic workloads for the forward-pass benchmarks and tests.

No public dataset is involved: each workload is specified by its sizes and
distributions, and every array here is drawn from ``numpy.random.default_rng``
with the given seed. X is float32 column-major (Fortran order), y is float32.

plain_fit         n=10,000 x p=2: x0~N(0,1), x1~Bernoulli(0.5),
                  y = 2 x0 + 3 x1 + x0 x1 + N(0,1); linear_only, max_terms=17.
hinge_search      n=100,000 x p=20 iid N(0,1); y = 6 random hinges
                  max(0, +-(x_j - t)) with t at a column quantile in [0.1, 0.9],
                  plus 3 products of two such hinges, coefficients U(-3,3),
                  noise N(0, 0.5^2); max_terms=31, max_degree=2, tail_span=0.
precision_stress  n=1,000,000 x p=100: 95 columns AR(1) across columns with
                  rho=0.9, plus 5 near-duplicates (a copy of a random earlier
                  column + N(0, (1e-4)^2)); y = sum over 5 disjoint column pairs
                  (a, b) of 2 x_a + 3 x_b + x_a x_b, + N(0,1); max_terms=63,
                  tail_span=0.
batched_fits      256 fits, n log-uniform in [1e3, 2e5], p uniform in [5, 50],
                  X iid N(0,1), y = 4 random hinges + N(0,1); max_terms=21.
"""
import hashlib

import numpy as np


def _fortran32(a):
    return np.asfortranarray(a.astype(np.float32))


def plain_fit(n=10_000, seed=0):
    rng = np.random.default_rng(seed)
    x0 = rng.standard_normal(n)
    x1 = rng.integers(0, 2, n).astype(np.float64)
    y = 2 * x0 + 3 * x1 + x0 * x1 + rng.standard_normal(n)
    X = _fortran32(np.stack([x0, x1], axis=1))
    kw = dict(max_terms=17, tail_span=0, linear_only=True)
    return X, y.astype(np.float32), kw


def _hinge(rng, X, j=None):
    n, p = X.shape
    if j is None:
        j = int(rng.integers(p))
    q = rng.uniform(0.1, 0.9)
    t = np.quantile(X[:, j], q)
    sign = 1.0 if rng.random() < 0.5 else -1.0
    return np.maximum(0.0, sign * (X[:, j].astype(np.float64) - t)), j


def hinge_search(n=100_000, p=20, seed=0, max_terms=31, noise=0.5):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, p))
    y = np.zeros(n)
    for _ in range(6):
        h, _j = _hinge(rng, X)
        y += rng.uniform(-3, 3) * h
    for _ in range(3):
        h1, j1 = _hinge(rng, X)
        j2 = (j1 + 1 + int(rng.integers(p - 1))) % p
        h2, _ = _hinge(rng, X, j2)
        y += rng.uniform(-3, 3) * h1 * h2
    y += noise * rng.standard_normal(n)
    kw = dict(max_terms=max_terms, max_degree=2, tail_span=0)
    return _fortran32(X), y.astype(np.float32), kw


def precision_stress(n=1_000_000, p=100, n_dup=5, rho=0.9, dup_std=1e-4, seed=0,
                     max_terms=63):
    rng = np.random.default_rng(seed)
    base = p - n_dup
    X = np.empty((n, p), dtype=np.float32, order="F")
    prev = rng.standard_normal(n)
    X[:, 0] = prev
    c = np.sqrt(1.0 - rho * rho)
    for j in range(1, base):
        prev = rho * prev + c * rng.standard_normal(n)
        X[:, j] = prev
    for j in range(base, p):
        src = int(rng.integers(base))
        X[:, j] = X[:, src] + dup_std * rng.standard_normal(n)
    cols = rng.choice(p, size=10, replace=False)
    y = np.zeros(n)
    for a, b in zip(cols[0::2], cols[1::2]):
        xa = X[:, a].astype(np.float64)
        xb = X[:, b].astype(np.float64)
        y += 2 * xa + 3 * xb + xa * xb
    y += rng.standard_normal(n)
    kw = dict(max_terms=max_terms, tail_span=0)
    return X, y.astype(np.float32), kw


def batched_fits(count=256, seed=0, n_lo=1_000, n_hi=200_000, p_lo=5, p_hi=50,
                 max_terms=21):
    """List of (X, y, kwargs), one per independent fit."""
    rng = np.random.default_rng(seed)
    fits = []
    for _ in range(count):
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        p = int(rng.integers(p_lo, p_hi + 1))
        X = rng.standard_normal((n, p))
        y = np.zeros(n)
        for _k in range(4):
            h, _j = _hinge(rng, X)
            y += rng.uniform(-3, 3) * h
        y += rng.standard_normal(n)
        fits.append((_fortran32(X), y.astype(np.float32),
                     dict(max_terms=max_terms, tail_span=0)))
    return fits


def batched_fits_top(k=4, count=256, seed=0):
    """The k fits of ``batched_fits(count, seed)`` with the largest n * p, in
    their order within the batch (the top of the n and p ranges)."""
    fits = batched_fits(count=count, seed=seed)
    order = sorted(range(len(fits)), key=lambda i: -fits[i][0].shape[0] * fits[i][0].shape[1])
    return [fits[i] for i in sorted(order[:k])]


def digest(*arrays):
    """sha256 over the raw bytes of the arrays (to pin generated inputs)."""
    h = hashlib.sha256()
    for a in arrays:
        a = np.asarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(np.ascontiguousarray(a).tobytes() if a.flags.c_contiguous
                 else np.asfortranarray(a).tobytes(order="F"))
    return h.hexdigest()


def knot_evals(n, endspan, min_span):
    """Grid cuts one (input, parent) candidate scores (marsalgo.cc:607-626):
    rows head+1, head+1+min_span, ... below n - endspan."""
    head = max(int(endspan), 0)
    tail = n - head
    first = head + 1
    if tail <= first:
        return 0
    return (tail - 1 - first) // min_span + 1
