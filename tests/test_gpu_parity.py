"""GPU parity: the CUDA path against the CPU oracle and the reference's goldens.

All calls go through the C ABI (include/mars_gpu.h) via mars_gb300.marslib.
The FP64 path reproduces the reference's scalar arithmetic operation for
operation (every reduction over rows is one fused chain in row order, every
reduction over basis columns one chain in column order), so against the
oracle -- the C restatement of that arithmetic -- it is compared for exact
equality: linear and hinge delta SSE, knots, append MSE, normalised columns,
squared norms and DGKS counts. Against the reference goldens (its x86 AVX
build, whose hinge reductions run in another order) the term path is exact and
r2 / r2_cv agree to 1e-6 (f4 fields).
"""
import numpy as np
import pytest

from mars_gb300 import mars
from tests import scenarios
from tests.golden import cases
from tests.test_oracle import assert_same_path, load_fit

pytestmark = pytest.mark.gpu

PRECISIONS = ["fp64"]


@pytest.fixture(scope="module")
def be_gpu(gpu):
    return scenarios.GpuBackend(precision="fp64")


@pytest.fixture(scope="module")
def be_port(port):
    return scenarios.OracleBackend("port")


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name", cases.FIT_CASES)
def test_golden_term_path_gpu(name, precision, gpu, monkeypatch):
    monkeypatch.setenv("MARS_GPU_PRECISION", precision)
    g = load_fit(name)
    X, y, w, kw = cases.fit_case(name)
    model = mars.fit(X, y, w, **kw)
    assert_same_path(model, g)


# How the FP64 sweep scores its cuts: "deferred" (partial scores stored, the ybx
# chain beside the sweep; steps whose partial scores stay under
# MARS_GPU_DEFER_BYTES) or "direct" (ybx first; the larger steps).
SCORING = {"deferred": None, "direct": "0"}


@pytest.mark.parametrize("scoring", sorted(SCORING))
@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name", cases.EVAL_CASES)
def test_eval_matches_oracle(name, precision, scoring, gpu, port, monkeypatch):
    import oracle

    if SCORING[scoring] is not None:
        monkeypatch.setenv("MARS_GPU_DEFER_BYTES", SCORING[scoring])

    X, y, w, appends, evals = cases.eval_case(name)
    a_gpu = gpu.MarsAlgo(X, y, w, cases.EVAL_MAX_TERMS)
    a_gpu.set_precision(precision)
    a_cpu = oracle.OracleAlgo(X, y, w, cases.EVAL_MAX_TERMS, kind="port")
    assert a_gpu.yvar() == a_cpu.yvar()
    for ap in appends:
        assert a_gpu.append(*ap) == a_cpu.append(*ap)
    assert a_gpu.nbasis() == a_cpu.nbasis()
    assert a_gpu.dsse() == a_cpu.dsse()
    for i, (ms, es, lo) in enumerate(evals):
        mask = cases.eval_mask(X.shape[1], a_cpu.nbasis(), i)
        dg, lg, hg, cg = a_gpu.eval(mask, ms, es, lo, 1)
        dc, lc, hc, cc = a_cpu.eval(mask, ms, es, lo, 1)
        assert dg == dc
        np.testing.assert_array_equal(lg, lc)
        np.testing.assert_array_equal(hg, hc)
        np.testing.assert_array_equal(cg, cc)
    mx, rss = a_gpu.orth_error()
    assert mx < 1e-5
    assert rss == pytest.approx(1 - a_gpu.dsse(), rel=1e-6)
    # the same figures for every leading basis: the last pair is the whole
    # basis', max |Q^T Q - I| only grows and the RSS only falls with the terms
    mk, rk = a_gpu.orth_error_by_terms()
    assert len(mk) == len(rk) == a_gpu.nbasis()
    assert (mk[-1], rk[-1]) == (mx, rss)
    assert np.all(np.diff(mk) >= 0) and np.all(np.diff(rk) <= 0)
    assert np.all(mk < 1e-5) and rk[0] <= 1.0


@pytest.mark.parametrize("name", ["hinge_search", "precision_stress_small", "weighted_nan"])
def test_golden_term_path_direct_scoring(name, gpu, monkeypatch):
    monkeypatch.setenv("MARS_GPU_PRECISION", "fp64")
    monkeypatch.setenv("MARS_GPU_DEFER_BYTES", "0")
    g = load_fit(name)
    X, y, w, kw = cases.fit_case(name)
    model = mars.fit(X, y, w, **kw)
    assert_same_path(model, g)


def test_delta_sse_gpu(be_gpu):
    scenarios.delta_sse(be_gpu, hinge_tol=1e-6)


def test_weighted_ls_gpu(be_gpu):
    scenarios.weighted_ls(be_gpu)


def test_min_span_gpu(be_gpu):
    scenarios.min_span(be_gpu)


def test_orthonormalize_basic_gpu(be_gpu):
    scenarios.orthonormalize_basic(be_gpu)


def test_orthonormalize_col_gpu(be_gpu):
    scenarios.orthonormalize_col_cases(be_gpu)


def test_orthonormalize_stress_matches_oracle(be_gpu, be_port):
    Bx_g, s_g, d_g = scenarios.orthonormalize_stress(be_gpu)
    Bx_c, s_c, d_c = scenarios.orthonormalize_stress(be_port)
    assert d_g == d_c
    np.testing.assert_array_equal(Bx_g, Bx_c)
    np.testing.assert_array_equal(s_g, s_c)


def test_orthonormalize_matches_oracle_random(be_gpu, be_port):
    rng = np.random.default_rng(5)
    n, m, p = 4096, 32, 12
    Bo = scenarios.make_orthonormal_basis(n, m, rng, bad_col=3)
    B = rng.uniform(-1, 1, (n, m)).astype(np.float32)
    B[:, 7] = B[:, 6]
    B[:, 10] = 0
    x = (rng.uniform(-1, 1, n) * 4).astype(np.float32)
    mask = np.sort(rng.permutation(m)[:p]).astype(np.int32)
    r_g = be_gpu.orthonormalize(np.asfortranarray(B), x, mask, Bo, m, 1e-14)
    r_c = be_port.orthonormalize(np.asfortranarray(B), x, mask, Bo, m, 1e-14)
    np.testing.assert_array_equal(r_g[0], r_c[0])
    np.testing.assert_array_equal(r_g[1], r_c[1])
    assert r_g[2] == r_c[2]


def _rand_problem(n, p, seed):
    rng = np.random.default_rng(seed)
    X = np.asfortranarray(rng.standard_normal((n, p)).astype(np.float32))
    y = (X[:, 0] - np.maximum(X[:, -1] - 0.3, 0) + 0.3 * rng.standard_normal(n)).astype(np.float32)
    return X, y, np.ones(n, np.float32)


def test_errors_match_reference_messages(gpu):
    X, y, w = _rand_problem(200, 3, 0)
    with pytest.raises(RuntimeError, match="target Y is all zero or NANs"):
        gpu.MarsAlgo(X, np.zeros(200, np.float32), w, 5)
    Xb = X.copy(order="F")
    Xb[7, 2] = np.nan
    with pytest.raises(RuntimeError, match="not all columns in X are finite"):
        gpu.MarsAlgo(Xb, y, w, 5)
    a = gpu.MarsAlgo(X, y, w, 2)
    with pytest.raises(RuntimeError, match="invalid basis column number: 1"):
        a.append("l", 0, 1, 0)
    with pytest.raises(RuntimeError, match="invalid basis type"):
        a.append("x", 0, 0, 0)
    with pytest.raises(RuntimeError, match="invalid dimension for mask"):
        a.eval(np.ones((3, 2), bool), 1, 0, False, 1)
    with pytest.raises(RuntimeError, match="min_span must be >= 1"):
        a.eval(np.ones((3, 1), bool), 0, 0, False, 1)
    with pytest.raises(RuntimeError, match="invalid X column index"):
        a.eval(np.ones((4, 1), bool), 1, 0, False, 1)
    assert a.append("l", 0, 0, 0) >= 0
    with pytest.raises(RuntimeError, match="basis matrix is full"):
        a.append("l", 1, 0, 0)


@pytest.mark.parametrize("end_span", [0, 1, 7, 199, 200, 5000])
def test_edge_end_span(gpu, port, end_span):
    import oracle

    X, y, w = _rand_problem(200, 3, 1)
    X[:, 1] = np.round(X[:, 1])  # ties
    a_g = gpu.MarsAlgo(X, y, w, 6)
    a_c = oracle.OracleAlgo(X, y, w, 6, kind="port")
    for ap in [("l", 0, 0, 0), ("+", 2, 0, 0.1)]:
        assert a_g.append(*ap) == a_c.append(*ap)
    mask = np.ones((3, a_c.nbasis()), bool)
    mask[2, 1] = False
    rg = a_g.eval(mask, 3, end_span, False, 1)
    rc = a_c.eval(mask, 3, end_span, False, 1)
    for k in (1, 2, 3):
        np.testing.assert_array_equal(rg[k], rc[k])


def test_edge_degenerate_columns(gpu, port):
    import oracle

    X, y, w = _rand_problem(300, 4, 2)
    X[:, 1] = 0.0          # all-zero column
    X[:, 2] = 1.5          # constant column (in the span of the intercept)
    a_g = gpu.MarsAlgo(X, y, w, 8)
    a_c = oracle.OracleAlgo(X, y, w, 8, kind="port")
    for ap in [("l", 1, 0, 0), ("l", 2, 0, 0), ("l", 0, 0, 0), ("-", 3, 0, 0.0)]:
        assert a_g.append(*ap) == a_c.append(*ap)
    assert a_g.nbasis() == a_c.nbasis()
    mask = np.ones((4, a_c.nbasis()), bool)
    mask[0, :] = False  # an input with no candidate
    rg = a_g.eval(mask, 1, 0, False, 1)
    rc = a_c.eval(mask, 1, 0, False, 1)
    for k in (1, 2, 3):
        np.testing.assert_array_equal(rg[k], rc[k])


def test_small_n_and_single_column(gpu, port):
    import oracle

    for n in (2, 3, 17):
        X, y, w = _rand_problem(n, 1, n)
        a_g = gpu.MarsAlgo(X, y, w, 4)
        a_c = oracle.OracleAlgo(X, y, w, 4, kind="port")
        mask = np.ones((1, 1), bool)
        rg = a_g.eval(mask, 1, 0, False, 1)
        rc = a_c.eval(mask, 1, 0, False, 1)
        for k in (1, 2, 3):
            np.testing.assert_array_equal(rg[k], rc[k])


def test_fit_with_weights_and_nan_target(gpu, port_lib):
    rng = np.random.default_rng(3)
    n = 3000
    X = np.asfortranarray(rng.standard_normal((n, 4)).astype(np.float32))
    y = (X[:, 0] * X[:, 1] + np.maximum(X[:, 2], 0) + 0.1 * rng.standard_normal(n)).astype(np.float32)
    y[::37] = np.nan
    w = (0.5 + rng.random(n)).astype(np.float32)
    kw = dict(max_terms=11, min_span=3, tail_span=0.01)
    m_g = mars.fit(X, y, w, **kw)
    m_c = mars.forward_pass(port_lib, X, y, w, **kw)
    def path(model):
        return [(r["type"], int(r["basis"]), int(r["input"]),
                 None if np.isnan(r["hinge"]) else float(r["hinge"])) for r in model]

    assert path(m_g) == path(m_c)


@pytest.mark.parametrize("defer", ["deferred", "direct"])
def test_wide_basis_matches_oracle(gpu, port, defer, monkeypatch):
    """More than 31 basis columns: the FP64 sweep then gives a candidate two
    component slots per lane, or, with few candidates, two warps. Bit-exact
    against the oracle either way, scored deferred or directly."""
    import oracle

    if defer == "direct":
        monkeypatch.setenv("MARS_GPU_DEFER_BYTES", "0")
    rng = np.random.default_rng(40)
    n, p = 3000, 6
    X, y, w = _rand_problem(n, p, 40)
    a_g = gpu.MarsAlgo(X, y, w, 48)
    a_c = oracle.OracleAlgo(X, y, w, 48, kind="port")
    for _ in range(400):
        if a_c.nbasis() >= 40:
            break
        j = int(rng.integers(p))
        b = int(rng.integers(a_c.nbasis()))
        t = float(X[int(rng.integers(n)), j])
        ap = ("+" if rng.random() < 0.5 else "-", j, b, t)
        assert a_g.append(*ap) == a_c.append(*ap)
    assert a_g.nbasis() == a_c.nbasis() >= 33
    m = a_c.nbasis()
    for cands in (3, 60):  # a few candidates (two warps each), then many (one warp)
        mask = np.zeros((p, m), bool)
        picks = rng.choice(p * m, size=cands, replace=False)
        mask.flat[picks] = True
        rg = a_g.eval(mask, 3, 2, False, 1)
        rc = a_c.eval(mask, 3, 2, False, 1)
        assert rg[0] == rc[0]
        for k in (1, 2, 3):
            np.testing.assert_array_equal(rg[k], rc[k])


# The column chains (norms of the projected columns, ybx, the norms of X) run
# either as written, one thread per chain (MARS_GPU_XCHAIN=0), or chunked over
# the rows with speculative runs and an exact walk (MARS_GPU_XCHAIN=1). Both
# must give the reference's values bit for bit.
XCHAIN = {"sequential": "0", "chunked": "1"}


@pytest.mark.parametrize("kernel", sorted(XCHAIN))
@pytest.mark.parametrize("name", cases.EVAL_CASES)
def test_column_chain_kernels_match_oracle(name, kernel, gpu, port, monkeypatch):
    import oracle

    monkeypatch.setenv("MARS_GPU_XCHAIN", XCHAIN[kernel])
    X, y, w, appends, evals = cases.eval_case(name)
    a_gpu = gpu.MarsAlgo(X, y, w, cases.EVAL_MAX_TERMS)
    a_cpu = oracle.OracleAlgo(X, y, w, cases.EVAL_MAX_TERMS, kind="port")
    assert a_gpu.yvar() == a_cpu.yvar()
    for ap in appends:
        assert a_gpu.append(*ap) == a_cpu.append(*ap)
    for i, (ms, es, lo) in enumerate(evals):
        mask = cases.eval_mask(X.shape[1], a_cpu.nbasis(), i)
        rg = a_gpu.eval(mask, ms, es, lo, 1)
        rc = a_cpu.eval(mask, ms, es, lo, 1)
        assert rg[0] == rc[0]
        for k in (1, 2, 3):
            np.testing.assert_array_equal(rg[k], rc[k])


@pytest.mark.parametrize("kernel", sorted(XCHAIN))
def test_column_chains_on_quantised_data(kernel, be_gpu, be_port, monkeypatch):
    """Quantised inputs make the chains' terms short dyadic numbers: long runs of
    exact sums and rounding ties, over n = 300,000 rows (160 chunks of 1,875)."""
    monkeypatch.setenv("MARS_GPU_XCHAIN", XCHAIN[kernel])
    rng = np.random.default_rng(41)
    n, m = 300_000, 6
    Bo = scenarios.make_orthonormal_basis(n, m, rng)
    B = (rng.integers(-32, 33, (n, m)) / 16).astype(np.float32)
    B[:, 0] = 1.0
    x = (rng.integers(-1024, 1025, n) / 64).astype(np.float32)
    mask = np.arange(m, dtype=np.int32)
    r_g = be_gpu.orthonormalize(np.asfortranarray(B), x, mask, Bo, m, 1e-14)
    r_c = be_port.orthonormalize(np.asfortranarray(B), x, mask, Bo, m, 1e-14)
    np.testing.assert_array_equal(r_g[0], r_c[0])
    np.testing.assert_array_equal(r_g[1], r_c[1])
    assert r_g[2] == r_c[2]


@pytest.mark.parametrize("kernel", sorted(XCHAIN))
def test_golden_term_path_chain_kernels(kernel, gpu, monkeypatch):
    monkeypatch.setenv("MARS_GPU_PRECISION", "fp64")
    monkeypatch.setenv("MARS_GPU_XCHAIN", XCHAIN[kernel])
    g = load_fit("hinge_search")
    X, y, w, kw = cases.fit_case("hinge_search")
    model = mars.fit(X, y, w, **kw)
    assert_same_path(model, g)
