"""Mixed precision (MARS_GPU_PREC_MIXED): every candidate ranked by the
FP32 / FP64-carry fast pass on the GPU, the best-ranked and the numerically
unreliable ones re-decided in the reference's exact FP64 order.

What it must keep: the decisions. The first maximum of the linear and of the
hinge delta SSE (mars.py:342-343), their values and the knot, are bit-exact
against the oracle, and the selected term sequence of every golden fit is the
reference's. Values of the other candidates are fast estimates held below the
best exact value, so they are not compared.
"""
import numpy as np
import pytest

from mars_gb300 import mars
from tests.golden import cases
from tests.test_oracle import assert_same_path, load_fit

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fallback", ["default", "never"])
@pytest.mark.parametrize("name", cases.FIT_CASES)
def test_mixed_golden_term_path(name, fallback, gpu, monkeypatch):
    """fallback 'never': every step through the fast pass, however many of
    its candidates need an exact re-decision."""
    monkeypatch.setenv("MARS_GPU_PRECISION", "mixed")
    if fallback == "never":
        monkeypatch.setenv("MARS_GPU_MIXED_FALLBACK", "2")
    g = load_fit(name)
    X, y, w, kw = cases.fit_case(name)
    model = mars.fit(X, y, w, **kw)
    assert_same_path(model, g)


def _first_max(a):
    j = int(np.argmax(a))
    return np.unravel_index(j, a.shape)


@pytest.mark.parametrize("name", cases.EVAL_CASES)
def test_mixed_eval_decisions_match_oracle(name, gpu, port):
    import oracle

    X, y, w, appends, evals = cases.eval_case(name)
    a_gpu = gpu.MarsAlgo(X, y, w, cases.EVAL_MAX_TERMS)
    a_gpu.set_precision("mixed")
    a_cpu = oracle.OracleAlgo(X, y, w, cases.EVAL_MAX_TERMS, kind="port")
    for ap in appends:
        assert a_gpu.append(*ap) == a_cpu.append(*ap)
    for i, (ms, es, lo) in enumerate(evals):
        mask = cases.eval_mask(X.shape[1], a_cpu.nbasis(), i)
        dg, lg, hg, cg = a_gpu.eval(mask, ms, es, lo, 1)
        dc, lc, hc, cc = a_cpu.eval(mask, ms, es, lo, 1)
        assert dg == dc
        jl = _first_max(lc)
        assert _first_max(lg) == jl
        assert lg[jl] == lc[jl]
        if not lo:
            jh = _first_max(hc)
            assert _first_max(hg) == jh
            assert hg[jh] == hc[jh]
            assert cg[jh] == cc[jh]
            # every other value is held strictly below the exact best
            assert np.all(hg[mask] <= hc[jh])
        assert np.all(lg[mask] <= lc[jl])
    st = a_gpu.stats()
    assert 0 < st["redecided"] <= st["candidates"]


def test_mixed_matches_fp64_on_a_fit_with_default_tail(gpu):
    """tail_span 0.02 (the reference default): the fast pass re-decides few
    candidates and the term path equals the FP64 path's."""
    from mars_gb300 import marslib
    from mars_gb300.mars import forward_pass
    from mars_gb300 import workloads

    X, y, kw = workloads.hinge_search(n=30_000, p=8, seed=3, max_terms=15)
    kw["tail_span"] = 0.02
    w = np.ones(len(y), np.float32)
    paths, stats = {}, {}
    for prec in ("fp64", "mixed"):
        hold = {}

        class Lib:
            __version__ = "0.12"

            def MarsAlgo(self, *a):
                o = marslib.MarsAlgo(*a)
                o.set_precision(prec)
                hold["a"] = o
                return o

        model = forward_pass(Lib(), X, y, w, threads=-1, **kw)
        paths[prec] = [(r["type"], int(r["basis"]), int(r["input"]), float(r["hinge"]))
                       for r in model]
        stats[prec] = hold["a"].stats()
    np.testing.assert_equal(paths["mixed"], paths["fp64"])
    assert stats["mixed"]["redecided"] < stats["mixed"]["candidates"] // 2


def test_rank_only_values_track_fp64(gpu, monkeypatch):
    """MARS_GPU_MIXED_RANK_ONLY=1 returns the fast values as they are (NaN cut
    where a candidate is flagged). Unflagged candidates within half of the best
    exact hinge score agree with the FP64 values to 1e-3 relative."""
    from mars_gb300 import marslib

    X, y, w, kw = cases.fit_case("hinge_search_small")
    if w is None:
        w = np.ones(len(y), np.float32)
    g = load_fit("hinge_search_small")
    mt = kw.get("max_terms", 31)
    out = {}
    for mode in ("fp64", "rank"):
        monkeypatch.setenv("MARS_GPU_MIXED_RANK_ONLY", "1" if mode == "rank" else "0")
        a = marslib.MarsAlgo(X, y, w, mt)
        a.set_precision("fp64" if mode == "fp64" else "mixed")
        for r in g["model"][1:9]:
            a.append(r["type"], int(r["input"]), int(r["basis"]),
                     float("nan") if r["hinge"] is None else r["hinge"])
        mask = np.ones((X.shape[1], a.nbasis()), bool)
        out[mode] = a.eval(mask, 6, 1, False, 1)
    _, l0, h0, _ = out["fp64"]
    _, l1, h1, c1 = out["rank"]
    flagged = np.isnan(c1)
    assert flagged.sum() < flagged.size
    ok = ~flagged & (h0 >= 0.5 * h0[~flagged].max())
    assert ok.any()
    np.testing.assert_allclose(h1[ok], h0[ok], rtol=1e-3)
    np.testing.assert_allclose(l1, l0, rtol=1e-3, atol=1e-9 * l0.max())
