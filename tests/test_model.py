"""Model surgery, storage and the backward elimination's host logic (CPU).

compact (mars.py:701-735) is checked on the reference's own scenarios
(tests/test_compact.py there, restated), dumps/loads on round trips. The
backward elimination (mars.py:547-695) is checked against the reference's
prune on the golden fixtures, with the Gram matrices computed here in FP64
(numpy) instead of on the GPU: on these well-conditioned bases that moves the
coefficients by ~1e-7 and leaves the selection unchanged. The GPU tests
(test_gpu_prune.py) run the whole prune, Gram matrices included, on every
fixture.
"""
import json
import os

import numpy as np
import pytest

from mars_gb300 import mars
from tests.golden import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _node(kind, basis=0, inp=0, hinge=np.nan):
    return (kind.encode(), basis, inp, hinge, 0, 0, 0, 0, 0)


def _model(nodes, beta):
    m = np.array(nodes, dtype=mars.MODEL_DTYPE)
    m["beta"] = beta
    return m


def test_compact_keeps_everything_when_nothing_is_pruned():
    m = _model([_node("i"), _node("l", 0, 0), _node("+", 1, 1, 3.0)], [1.0, 2.0, 3.0])
    c = mars.compact(m)
    assert len(c) == 3
    np.testing.assert_array_equal(c["beta"], [1.0, 2.0, 3.0])


def test_compact_drops_a_pruned_leaf():
    m = _model([_node("i"), _node("l", 0, 0), _node("l", 0, 1)], [1.0, 2.0, 0.0])
    c = mars.compact(m)
    assert len(c) == 2 and list(c["input"]) == [0, 0]


def test_compact_keeps_a_pruned_parent_of_a_kept_child():
    m = _model([_node("i"), _node("l", 0, 0), _node("+", 1, 1, 0.5), _node("l", 0, 2)],
               [1.0, 0.0, 2.0, 0.0])
    c = mars.compact(m)
    assert len(c) == 3
    assert c[2]["basis"] == 1 and c[1]["beta"] == 0.0


def test_compact_remaps_parent_indices():
    m = _model([_node("i"), _node("l", 0, 0), _node("l", 0, 1), _node("+", 2, 2, 0.1),
                _node("-", 2, 2, 0.1)], [1.0, 0.0, 1.0, 0.0, 3.0])
    c = mars.compact(m)
    assert [int(r["basis"]) for r in c] == [0, 0, 1]
    assert [r["type"] for r in c] == [b"i", b"l", b"-"]


def test_compact_keeps_a_whole_chain_for_its_leaf():
    m = _model([_node("i"), _node("l", 0, 0), _node("l", 1, 1), _node("l", 2, 2)],
               [0.0, 0.0, 0.0, 5.0])
    c = mars.compact(m)
    assert len(c) == 4
    np.testing.assert_array_equal(c["beta"], [0.0, 0.0, 0.0, 5.0])


def test_compact_everything_pruned():
    assert len(mars.compact(_model([_node("i"), _node("l", 0, 0)], [0.0, 0.0]))) == 0


def test_compact_predicts_the_same():
    rng = np.random.default_rng(7)
    X = rng.standard_normal((50, 3)).astype(np.float32)
    m = _model([_node("i"), _node("l", 0, 0), _node("l", 0, 1), _node("+", 1, 2, 0.5)],
               [2.0, 3.0, 0.0, -1.0])
    c = mars.compact(m)
    np.testing.assert_allclose(mars.expand(X, c) @ c["beta"], mars.expand(X, m) @ m["beta"],
                               atol=1e-6)


def test_dumps_loads_round_trip(tmp_path):
    g = json.load(open(os.path.join(GOLDEN, "hinge_search.json")))
    m = cases.model_from_rows(g["model"])
    m["beta"] = np.arange(len(m), dtype=np.float32)
    back = mars.loads(mars.dumps(m))
    assert back.dtype == mars.MODEL_DTYPE
    assert back.tobytes() == m.tobytes()
    path = tmp_path / "model.npy"
    mars.save(str(path), m)
    assert mars.load(str(path)).tobytes() == m.tobytes()
    # the file is a plain .npy of the structured array
    assert np.load(str(path), allow_pickle=False).tobytes() == m.tobytes()


def test_loads_rejects_other_arrays():
    import io

    buf = io.BytesIO()
    np.save(buf, np.zeros(3))
    with pytest.raises(ValueError, match="not a MARS model"):
        mars.loads(buf.getvalue())


def _numpy_gram(A, B=None):
    if B is None:
        B = A
    A = np.asarray(A)
    B = np.asarray(B)
    A2 = A.reshape(len(A), -1) if A.ndim == 1 else A
    B2 = B.reshape(len(B), -1) if B.ndim == 1 else B
    out = A2.astype(np.float64).T @ B2.astype(np.float64)
    if A.ndim == 1 and B.ndim == 1:
        return float(out[0, 0])
    if A.ndim == 1:
        return out[0]
    if B.ndim == 1:
        return out[:, 0]
    return out


@pytest.mark.parametrize("fit", ["precision_stress_small", "weighted_nan"])
def test_elimination_matches_reference_prune(fit, monkeypatch):
    monkeypatch.setattr(mars, "gram", _numpy_gram)
    ref = np.load(os.path.join(GOLDEN, "prune_%s.npz" % fit))
    rows = json.load(open(os.path.join(GOLDEN, fit + ".json")))["model"]
    X, y, w, _ = cases.fit_case(fit)
    model = cases.model_from_rows(rows)
    B = mars.expand(X, model)
    for tag, kw in cases.prune_variants(len(model)):
        beta = mars.prune(B, y, w, **kw)
        want = ref["beta_" + tag]
        np.testing.assert_array_equal(beta != 0, want != 0)
        np.testing.assert_allclose(beta, want, rtol=0, atol=1e-5 * np.abs(want).max())


def test_elimination_scenarios_match_reference_prune(monkeypatch):
    monkeypatch.setattr(mars, "gram", _numpy_gram)
    ref = np.load(os.path.join(GOLDEN, "prune_scenarios.npz"))
    for i, (B, y, w, kw) in enumerate(cases.prune_scenarios()):
        beta = mars.prune(B, y, w, **kw)
        want = ref["beta_%d" % i]
        np.testing.assert_array_equal(beta != 0, want != 0)
        np.testing.assert_allclose(beta, want, rtol=1e-9, atol=1e-9)
