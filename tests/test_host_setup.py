"""The fit's set-up on the host (mars_gb300/csrc/host_exact.cpp,
marsalgo.cc:266-370) without a GPU: compiled on its own with the library's
host flags and checked against the oracle port, which follows the reference's
constructor. yvar and y . intercept must agree bit for bit; the scaled target,
intercept and column scales to a few ulps of a float64 restatement; invalid
input raises the reference's messages."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "mars_gb300", "csrc")


@pytest.fixture(scope="module")
def hs(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("host_setup") / "host_setup.so")
    subprocess.run(["g++", "-O3", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
                    "-pthread", "-I", CSRC, "-o", out, os.path.join(HERE, "host_setup.cpp"),
                    os.path.join(CSRC, "host_exact.cpp")], check=True)
    lib = ctypes.CDLL(out)
    fp = ctypes.POINTER(ctypes.c_float)
    dp = ctypes.POINTER(ctypes.c_double)
    sz = ctypes.c_size_t
    lib.hs_init.restype = ctypes.c_int
    lib.hs_init.argtypes = [fp, fp, fp, sz, sz, sz, dp, dp, dp, fp, fp, fp, ctypes.c_char_p,
                            ctypes.c_int]
    return lib


@pytest.fixture(scope="module")
def port():
    if not oracle.available("port"):
        oracle.build(with_reference=False)
    return oracle


def setup(lib, X, y, w):
    X = np.asfortranarray(X, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    w = np.ascontiguousarray(w, np.float32)
    n, p = X.shape
    fp = ctypes.POINTER(ctypes.c_float)
    yvar, ybo0, tol = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    s, yn, b0 = np.zeros(p, np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)
    err = ctypes.create_string_buffer(256)
    rc = lib.hs_init(X.ctypes.data_as(fp), y.ctypes.data_as(fp), w.ctypes.data_as(fp), n, p, n,
                     ctypes.byref(yvar), ctypes.byref(ybo0), ctypes.byref(tol),
                     s.ctypes.data_as(fp), yn.ctypes.data_as(fp), b0.ctypes.data_as(fp), err, 256)
    if rc:
        raise RuntimeError(err.value.decode())
    return yvar.value, ybo0.value, tol.value, s, yn, b0


def problems():
    r = np.random.default_rng(5)
    n, p = 5000, 7
    X = r.standard_normal((n, p)).astype(np.float32) * np.float32(3.0)
    X[:, 3] = 0.0  # a constant-zero column keeps scale 1
    y = (X[:, 0] * 2 + r.standard_normal(n)).astype(np.float32)
    yield "plain", X, y, np.ones(n, np.float32)
    w = r.uniform(0.1, 4.0, n).astype(np.float32)
    yield "weighted", X, y, w
    y2 = y.copy()
    y2[::17] = np.nan  # non-finite targets get weight 0
    yield "nan_targets", X, y2, w
    X1 = np.empty((1, p), np.float32, order="F")  # unit row stride, as the binding wants
    X1[:] = X[:1]
    yield "one_row", X1, y[:1], w[:1]


@pytest.mark.parametrize("case", range(4))
def test_setup_matches_oracle(hs, port, case):
    name, X, y, w = list(problems())[case]
    X = np.asfortranarray(X)
    yvar, ybo0, tol, s, yn, b0 = setup(hs, X, y, w)
    ref = port.OracleAlgo(X, y, w, 5, kind="port")
    assert yvar == ref.yvar(), name
    assert ybo0 * ybo0 == ref.dsse(), name  # fma(ybo0, ybo0, 0): one rounding
    n = X.shape[0]
    assert tol == (n * 0.02) * np.finfo(np.float64).eps
    # float64 restatements (numpy's own summation order: a few ulps)
    sw = np.sqrt(w.astype(np.float64))
    yd = y.astype(np.float64) * sw
    bad = ~np.isfinite(yd)
    yd[bad], sw[bad] = 0.0, 0.0
    np.testing.assert_allclose(yn, (yd / np.linalg.norm(yd)).astype(np.float32), rtol=2e-7,
                               atol=1e-30)
    np.testing.assert_allclose(b0, (sw / np.linalg.norm(sw)).astype(np.float32), rtol=2e-7,
                               atol=1e-30)
    rms = np.sqrt((X.astype(np.float64) ** 2).mean(0))
    want = np.where(rms > 0, 1.0 / np.where(rms > 0, rms, 1.0), 1.0).astype(np.float32)
    np.testing.assert_allclose(s, want, rtol=2e-7)
    assert s[3] == 1.0


def test_setup_errors(hs):
    r = np.random.default_rng(6)
    X = r.standard_normal((100, 3)).astype(np.float32)
    w = np.ones(100, np.float32)
    with pytest.raises(RuntimeError, match="target Y is all zero or NANs"):
        setup(hs, X, np.zeros(100, np.float32), w)
    with pytest.raises(RuntimeError, match="target Y is all zero or NANs"):
        setup(hs, X, np.full(100, np.nan, np.float32), w)
    X2 = X.copy()
    X2[7, 1] = np.inf
    with pytest.raises(RuntimeError, match="not all columns in X are finite"):
        setup(hs, X2, r.standard_normal(100).astype(np.float32), w)
