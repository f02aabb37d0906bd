"""The library's host-side append (mars_gb300/csrc/host_exact.cpp) on CPU.

For long columns an append (marsalgo.cc:760-875, kernels.cc:194-281) splits its
elementwise loops over a pool of host threads, and on request
(MARS_GPU_HOST_XCHAIN=1) runs its serial FP64 chains chunked with the exact
speculation. These tests run the same appends in order and over the pool
(MARS_GPU_HOST_PAR_ROWS) and require identical bits, and MSEs equal to the
oracle port's.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def hlib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("host_append") / "host_append.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
                    "-pthread", "-o", out, os.path.join(HERE, "host_append_harness.cpp"),
                    os.path.join(ROOT, "mars_gb300", "csrc", "host_exact.cpp")], check=True)
    lib = ctypes.CDLL(out)
    fp = ctypes.POINTER(ctypes.c_float)
    lib.ha_create.restype = ctypes.c_void_p
    lib.ha_create.argtypes = [fp, fp, fp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t]
    lib.ha_append.restype = ctypes.c_double
    lib.ha_append.argtypes = [ctypes.c_void_p, ctypes.c_char, ctypes.c_int, ctypes.c_int,
                              ctypes.c_float, ctypes.POINTER(ctypes.c_long)]
    lib.ha_nbasis.restype = ctypes.c_size_t
    lib.ha_nbasis.argtypes = [ctypes.c_void_p]
    lib.ha_column.argtypes = [ctypes.c_void_p, ctypes.c_int, fp, fp]
    lib.ha_ybo.restype = ctypes.c_double
    lib.ha_ybo.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.ha_bo_row.argtypes = [ctypes.c_void_p, ctypes.c_size_t, fp]
    lib.ha_destroy.argtypes = [ctypes.c_void_p]
    return lib


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def problem(n, p, seed):
    r = np.random.default_rng(seed)
    X = np.asfortranarray(r.standard_normal((n, p)).astype(np.float32))
    y = (2 * X[:, 0] + np.maximum(X[:, 1] - 0.3, 0) + r.standard_normal(n)).astype(np.float32)
    return X, y, np.ones(n, np.float32)


def appends(p, count, seed, X):
    r = np.random.default_rng(seed)
    out, m = [], 1
    for k in range(count):
        t = "l+-"[k % 3]
        j = int(r.integers(p))
        b = int(r.integers(m))
        h = float(X[int(r.integers(X.shape[0])), j])
        out.append((t, j, b, h))
        m += 1
    return out


def run_appends(lib, X, y, w, aps, max_terms, par_rows, monkeypatch, chunked=False):
    monkeypatch.setenv("MARS_GPU_HOST_PAR_ROWS", str(par_rows))
    monkeypatch.setenv("MARS_GPU_HOST_XCHAIN", "1" if chunked else "0")
    n, p = X.shape
    h = lib.ha_create(_fp(X), _fp(y), _fp(w), n, p, max_terms)
    mses, dg = [], ctypes.c_long(0)
    for t, j, b, hh in aps:
        if b >= lib.ha_nbasis(h):
            b = 0
        mses.append(lib.ha_append(h, t.encode(), j, b, hh, ctypes.byref(dg)))
    m = lib.ha_nbasis(h)
    cols = np.empty((m, n), np.float32)
    bcols = np.empty((m, n), np.float32)
    for j in range(m):
        lib.ha_column(h, j, _fp(cols[j]), _fp(bcols[j]))
    ybo = [lib.ha_ybo(h, j) for j in range(m)]
    rows = np.empty((3, max_terms), np.float32)
    for q, i in enumerate((0, n // 2, n - 1)):
        lib.ha_bo_row(h, i, _fp(rows[q]))
    lib.ha_destroy(h)
    return np.array(mses), cols, bcols, np.array(ybo), dg.value, rows


@pytest.mark.parametrize("chunked", [False, True])
@pytest.mark.parametrize("n", [1, 37, 5000, 300_000])
def test_pool_appends_equal_in_order(hlib, n, chunked, monkeypatch):
    X, y, w = problem(n, 6, 11)
    aps = appends(6, 14, 12, X)
    seq = run_appends(hlib, X, y, w, aps, 20, 10 ** 12, monkeypatch)
    par = run_appends(hlib, X, y, w, aps, 20, 0, monkeypatch, chunked)
    assert seq[0].view(np.uint64).tolist() == par[0].view(np.uint64).tolist()
    np.testing.assert_array_equal(seq[1].view(np.uint32), par[1].view(np.uint32))
    np.testing.assert_array_equal(seq[2].view(np.uint32), par[2].view(np.uint32))
    assert seq[3].view(np.uint64).tolist() == par[3].view(np.uint64).tolist()
    assert seq[4] == par[4]
    np.testing.assert_array_equal(seq[5].view(np.uint32), par[5].view(np.uint32))


@pytest.mark.parametrize("chunked", [False, True])
def test_pool_appends_equal_oracle(hlib, chunked, monkeypatch):
    import oracle

    n, p = 300_000, 5
    X, y, w = problem(n, p, 13)
    aps = appends(p, 10, 14, X)
    got = run_appends(hlib, X, y, w, aps, 16, 0, monkeypatch, chunked)[0]
    a = oracle.OracleAlgo(X, y, w, 16, kind="port")
    want = []
    for t, j, b, hh in aps:
        if b >= a.nbasis():
            b = 0
        want.append(a.append(t, j, b, hh))
    assert np.array(want).view(np.uint64).tolist() == got.view(np.uint64).tolist()


def test_pool_appends_with_dgks(hlib, monkeypatch):
    """Near-dependent columns make the DGKS re-projection fire; duplicated
    columns are rejected (-1). In order and over the pool alike."""
    n = 280_000
    X, y, w = problem(n, 3, 15)
    X[:, 2] = X[:, 1] * np.float32(1.0000001)
    aps = [("l", 1, 0, 0.0), ("l", 2, 0, 0.0), ("+", 1, 0, 0.2), ("+", 2, 0, 0.2),
           ("-", 0, 1, 0.1), ("-", 0, 2, 0.1), ("l", 1, 0, 0.0)]
    seq = run_appends(hlib, X, y, w, aps, 12, 10 ** 12, monkeypatch)
    for chunked in (False, True):
        par = run_appends(hlib, X, y, w, aps, 12, 0, monkeypatch, chunked)
        assert seq[0].view(np.uint64).tolist() == par[0].view(np.uint64).tolist()
        assert seq[4] == par[4]
    assert (seq[0] == -1).any()
