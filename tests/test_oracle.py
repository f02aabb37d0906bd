"""Pins the CPU oracle (the C restatement) to the reference.

* term paths and eval vectors produced by the reference itself
  (tests/golden/, written by tests/golden/make_golden.py);
* bit-exactness against the reference sources compiled without their AVX
  branches (only where oracle/_ref/ was built, i.e. next to the reference);
* the reference's own unit-test scenarios and tolerances (tests/scenarios.py).
"""
import json
import os

import numpy as np
import pytest

from mars_gb300 import workloads
from mars_gb300.mars import forward_pass
from tests import scenarios
from tests.golden import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_fit(name):
    path = os.path.join(GOLDEN, name + ".json")
    if name in cases.LARGE_CASES and not os.path.isfile(path):
        pytest.skip("fixture %s not generated" % name)
    with open(path) as f:
        return json.load(f)


def assert_same_path(model, golden, r2_tol=1e-6):
    rows = golden["model"]
    got = [(r["type"].decode(), int(r["basis"]), int(r["input"]),
            None if np.isnan(r["hinge"]) else float(r["hinge"])) for r in model]
    want = [(r["type"], r["basis"], r["input"], r["hinge"]) for r in rows]
    assert got == want
    np.testing.assert_allclose(model["r2"], [r["r2"] for r in rows], rtol=0, atol=r2_tol)
    np.testing.assert_allclose(model["r2_cv"], [r["r2_cv"] for r in rows], rtol=0, atol=r2_tol)
    assert [int(r["order"]) for r in model] == [r["order"] for r in rows]


@pytest.mark.parametrize("name", [c for c in cases.FIT_CASES if c not in cases.LARGE_CASES])
def test_golden_term_path(name, port_lib):
    g = load_fit(name)
    X, y, w, kw = cases.fit_case(name)
    digest = workloads.digest(X, y) if w is None else workloads.digest(X, y, w)
    assert digest == g["digest"], "input generator changed; regenerate tests/golden"
    model = forward_pass(port_lib, X, y, w, threads=-1, **kw)
    assert_same_path(model, g)


@pytest.mark.parametrize("name", cases.LARGE_CASES)
def test_large_golden_inputs_unchanged(name):
    """The large fixtures (hours of reference CPU time; the GPU tests fit
    them) still describe the inputs the generators make."""
    if not os.path.isfile(os.path.join(GOLDEN, name + ".json")):
        pytest.skip("fixture %s not generated" % name)
    g = load_fit(name)
    X, y, w, kw = cases.fit_case(name)
    assert workloads.digest(X, y) == g["digest"], "input generator changed; regenerate"
    assert g["kwargs"] == kw
    assert len(g["model"]) >= 2


def test_largest_batched_fits_term_paths(port_lib):
    """The port gives the reference's term paths on the four largest of the
    256 batched fits (n 1.6-1.8e5, p 40-47; ~10 s of CPU each)."""
    names = [c for c in cases.LARGE_CASES if c.startswith("batched_top_")]
    fits = workloads.batched_fits_top(k=len(names))
    for name, (X, y, kw) in zip(names, fits):
        g = load_fit(name)
        assert workloads.digest(X, y) == g["digest"], name
        model = forward_pass(port_lib, X, y, None, threads=-1, **kw)
        assert_same_path(model, g)


@pytest.mark.parametrize("name", cases.EVAL_CASES)
def test_golden_eval_vectors(name, port):
    import oracle

    ref = np.load(os.path.join(GOLDEN, name + ".npz"))
    X, y, w, appends, evals = cases.eval_case(name)
    assert workloads.digest(X, y, w) == str(ref["digest"])
    algo = oracle.OracleAlgo(X, y, w, cases.EVAL_MAX_TERMS, kind="port")
    mses = [algo.append(*a) for a in appends]
    np.testing.assert_allclose(mses, ref["mses"], rtol=1e-12)
    assert algo.nbasis() == int(ref["nbasis"])
    assert algo.yvar() == pytest.approx(float(ref["yvar"]), rel=1e-14)
    for i, (ms, es, lo) in enumerate(evals):
        mask = cases.eval_mask(X.shape[1], algo.nbasis(), i)
        d, lin, hin, cut = algo.eval(mask, ms, es, lo, 2)
        assert d == pytest.approx(float(ref["dsse_%d" % i]), rel=1e-14)
        np.testing.assert_allclose(lin, ref["lin_%d" % i], rtol=1e-10, atol=1e-300)
        # The fixtures come from the reference's AVX build; its f/g reduction
        # order differs from the scalar branch restated here, which moves the
        # ill-conditioned cuts by ~1e-7 relative (unittest.cc:9-21).
        np.testing.assert_allclose(hin, ref["hin_%d" % i], rtol=1e-6, atol=1e-300)
        np.testing.assert_array_equal(cut, ref["cut_%d" % i])


needs_ref = pytest.mark.skipif(
    not os.path.isfile(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                    "libmars_ref_scalar.so")),
    reason="reference build not present (only where the reference sources are)")


@needs_ref
@pytest.mark.parametrize("name", cases.EVAL_CASES)
def test_port_bitexact_vs_reference_scalar(name, port):
    import oracle

    X, y, w, appends, evals = cases.eval_case(name)
    algos = [oracle.OracleAlgo(X, y, w, cases.EVAL_MAX_TERMS, kind=k)
             for k in ("port", "ref_scalar")]
    for a in appends:
        m0, m1 = algos[0].append(*a), algos[1].append(*a)
        assert m0 == pytest.approx(m1, rel=4e-16, abs=0)
    for i, (ms, es, lo) in enumerate(evals):
        mask = cases.eval_mask(X.shape[1], algos[0].nbasis(), i)
        r0 = algos[0].eval(mask, ms, es, lo, 3)
        r1 = algos[1].eval(mask, ms, es, lo, 3)
        for a0, a1 in zip(r0[1:], r1[1:]):
            np.testing.assert_array_equal(a0, a1)


def test_argsort_stable_descending(port):
    rng = np.random.default_rng(3)
    v = np.round(rng.standard_normal(5000) * 4).astype(np.float32) / 4
    v[::97] = -0.0
    v[::89] = 0.0
    k = port.k_argsort(v)
    np.testing.assert_array_equal(k, np.argsort(-v, kind="stable"))


def test_covariates_matches_definition(port):
    """unittest.cc:166-209: f += k0 g; g += k1 x; ff = f.f; fy = f.y."""
    import ctypes

    rng = np.random.default_rng(4)
    n, m = 809, 131
    X = rng.uniform(-1, 1, (n, m)).astype(np.float32)
    y = rng.uniform(-1, 1, m)
    K = rng.uniform(-1, 1, (n, 4)).astype(np.float32)
    f0 = np.zeros(m + 1)
    g0 = np.zeros(m + 1)
    f1 = np.zeros(m + 1)
    g1 = np.zeros(m + 1)
    dp = ctypes.POINTER(ctypes.c_double)
    for i in range(n):
        ff, fy = ctypes.c_double(), ctypes.c_double()
        row = np.ascontiguousarray(X[i])
        port.covariates(f0.ctypes.data_as(dp), g0.ctypes.data_as(dp),
                        row.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                        y.ctypes.data_as(dp), float(K[i, 0]), float(K[i, 1]), float(K[i, 2]),
                        float(K[i, 3]), m, ctypes.byref(ff), ctypes.byref(fy))
        f1 += float(K[i, 2]) * g1
        g1[:m] += float(K[i, 3]) * row.astype(np.float64)
        g1[m] += float(K[i, 3]) * float(K[i, 0])
        ff1 = float(f1 @ f1)
        fy1 = float(f1[:m] @ y + f1[m] * float(K[i, 1]))
        assert np.linalg.norm(f0 - f1) < 1e-9 and np.linalg.norm(g0 - g1) < 1e-9
        if ff1 > 0:
            assert ff.value / ff1 == pytest.approx(1, abs=1e-6)
        if fy1 > 0:
            assert fy.value / fy1 == pytest.approx(1, abs=1e-6)


@pytest.fixture(scope="module")
def be(port):
    return scenarios.OracleBackend("port")


def test_delta_sse(be):
    # the oracle restates the reference's scalar path: HINGE_DSSE_TOL = 1e-5
    scenarios.delta_sse(be, hinge_tol=1e-5)


def test_weighted_ls(be):
    scenarios.weighted_ls(be)


def test_min_span(be):
    scenarios.min_span(be)


def test_orthonormalize_basic(be):
    scenarios.orthonormalize_basic(be)


def test_orthonormalize_precision_stress(be):
    scenarios.orthonormalize_stress(be)


def test_orthonormalize_col(be):
    scenarios.orthonormalize_col_cases(be)


def test_oracle_errors(port_lib):
    import oracle

    rng = np.random.default_rng(0)
    X = np.asfortranarray(rng.standard_normal((100, 3)).astype(np.float32))
    with pytest.raises(RuntimeError, match="target Y is all zero or NANs"):
        oracle.OracleAlgo(X, np.zeros(100, np.float32), np.ones(100, np.float32), 5)
    Xb = X.copy(order="F")
    Xb[3, 1] = np.inf
    with pytest.raises(RuntimeError, match="not all columns in X are finite"):
        oracle.OracleAlgo(Xb, np.ones(100, np.float32), np.ones(100, np.float32), 5)
    a = oracle.OracleAlgo(X, rng.standard_normal(100).astype(np.float32),
                          np.ones(100, np.float32), 2)
    with pytest.raises(RuntimeError, match="invalid basis column number: 3"):
        a.append("l", 0, 3, 0)
    assert a.append("l", 0, 0, 0) >= 0
    with pytest.raises(RuntimeError, match="basis matrix is full"):
        a.append("l", 1, 0, 0)
