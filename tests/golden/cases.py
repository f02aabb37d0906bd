"""Definitions of the golden cases, shared by make_golden.py and the tests.

Fit cases run the whole forward pass (``fit``) and pin the selected term
sequence. Eval cases pin one ``MarsAlgo`` state after a fixed series of
``append`` calls and the (linear, hinge, cut) outputs of ``eval`` on it.
"""
import numpy as np

from mars_gb300 import workloads

FIT_CASES = [
    "plain_fit",
    "hinge_search",
    "hinge_search_small",
    "precision_stress_small",
    "weighted_nan",
    "fastmars_caps",
    "batched_small_0",
    "batched_small_1",
    "batched_small_2",
    "default_tail",
    "precision_stress",
    "precision_stress_tail0",
    "batched_top_0",
    "batched_top_1",
    "batched_top_2",
    "batched_top_3",
]
# Fixtures that take minutes to hours of reference CPU time; the tests that
# need them skip when they are absent.
LARGE_CASES = ["precision_stress", "precision_stress_tail0", "batched_top_0", "batched_top_1",
               "batched_top_2", "batched_top_3"]
EVAL_CASES = ["eval_planted_knot", "eval_ties"]
# Backward-pass (prune) fixtures: the reference's prune on the expanded golden
# models, and on small scenarios.
PRUNE_MODEL_CASES = ["hinge_search", "precision_stress_small", "weighted_nan"]
PRUNE_CASES = ["prune_" + c for c in PRUNE_MODEL_CASES] + ["prune_scenarios"]
EVAL_MAX_TERMS = 16


def fit_case(name):
    """(X, y, w or None, fit kwargs) for a fit case."""
    w = None
    if name == "plain_fit":
        X, y, kw = workloads.plain_fit()
    elif name == "hinge_search":
        X, y, kw = workloads.hinge_search()
    elif name == "hinge_search_small":
        X, y, kw = workloads.hinge_search(n=20_000, p=8, seed=3, max_terms=15)
    elif name == "precision_stress_small":
        X, y, kw = workloads.precision_stress(n=30_000, p=20, n_dup=3, seed=5, max_terms=21)
    elif name == "weighted_nan":
        rng = np.random.default_rng(11)
        n, p = 5000, 5
        X = rng.standard_normal((n, p))
        y = X[:, 1] * 0.5 - np.maximum(X[:, 2] - 0.3, 0) + 0.1 * rng.standard_normal(n)
        y[rng.integers(0, n, 25)] = np.nan
        w = (0.01 + 10.0 * np.abs(X[:, 0])).astype(np.float32)
        X = np.asfortranarray(X.astype(np.float32))
        y = y.astype(np.float32)
        kw = dict(max_terms=11, max_degree=2)
    elif name == "fastmars_caps":
        X, y, _ = workloads.hinge_search(n=8000, p=12, seed=7, max_terms=15)
        kw = dict(max_terms=15, max_basis=3, max_inputs=4, self_interact=True, min_span=5,
                  tail_span=0.01)
    elif name.startswith("batched_small_"):
        k = int(name.rsplit("_", 1)[1])
        fits = workloads.batched_fits(count=3, seed=4, n_hi=20_000, p_hi=12)
        X, y, kw = fits[k]
    elif name == "precision_stress":
        # the full precision-stress workload at the reference's default tail span
        X, y, kw = workloads.precision_stress()
        kw["tail_span"] = 0.02
    elif name == "precision_stress_tail0":
        # the same workload with cuts scored down to the last rows (tail_span 0)
        X, y, kw = workloads.precision_stress()
    elif name.startswith("batched_top_"):
        k = int(name.rsplit("_", 1)[1])
        X, y, kw = workloads.batched_fits_top(4)[k]
    elif name == "default_tail":
        X, y, _ = workloads.hinge_search(n=12_000, p=6, seed=9)
        kw = dict(max_terms=13)
    else:
        raise KeyError(name)
    return X, y, w, kw


def eval_case(name):
    """(X, y, w, appends, evals) for an eval case. evals: (min_span, endspan, linear_only)."""
    if name == "eval_planted_knot":
        rng = np.random.default_rng(21)
        n, p = 3000, 8
        X = rng.uniform(-1, 1, (n, p))
        X[100, 7] = 0.25
        X[:, 6] = 0.0
        y = (0.3 * X[:, 3] - 0.2 * X[:, 5] + 0.25 * X[:, 3] * X[:, 5]
             - 5 * np.maximum(X[:, 7] - 0.25, 0) + 2 * np.maximum(0.25 - X[:, 7], 0)
             + rng.uniform(-1, 1, n))
        appends = [("l", 3, 0, 0.0), ("l", 5, 0, 0.0), ("l", 5, 1, 0.0),
                   ("+", 7, 0, 0.25), ("-", 7, 0, 0.25)]
        evals = [(1, 0, False), (3, 5, False), (1, 0, True), (7, 50, False)]
    elif name == "eval_ties":
        rng = np.random.default_rng(22)
        n, p = 2500, 5
        X = rng.standard_normal((n, p))
        X[:, 2] = np.round(X[:, 2] * 2) / 2     # heavy ties
        X[:, 4] = (rng.random(n) < 0.5)         # binary
        y = (X[:, 0] + np.maximum(X[:, 2] - 0.5, 0) - X[:, 1] * X[:, 4]
             + 0.2 * rng.standard_normal(n))
        appends = [("l", 0, 0, 0.0), ("+", 2, 0, 0.5), ("-", 2, 0, 0.5), ("l", 4, 0, 0.0),
                   ("l", 1, 4, 0.0)]
        evals = [(1, 0, False), (2, 3, False), (4, 1, True)]
    else:
        raise KeyError(name)
    X = np.asfortranarray(X.astype(np.float32))
    y = y.astype(np.float32)
    w = np.ones(len(y), dtype=np.float32)
    return X, y, w, appends, evals


def eval_mask(p, m, i):
    """Deterministic (p, m) mask for the i-th eval of a case: all true except a
    fixed pattern of holes (and one fully masked row) so masking is exercised."""
    mask = np.ones((p, m), dtype=bool)
    if i % 2 == 1:
        mask[1, :] = False
        mask[:, m // 2] = False
        mask[p - 1, 0] = False
    return mask


def model_from_rows(rows):
    """The model array (the forward pass's dtype) from a fit fixture's rows."""
    from mars_gb300.mars import MODEL_DTYPE

    model = np.zeros(len(rows), dtype=MODEL_DTYPE)
    for i, r in enumerate(rows):
        model[i] = (r["type"].encode(), r["basis"], r["input"],
                    np.nan if r["hinge"] is None else r["hinge"], np.nan, r["r2"],
                    r["r2_cv"], r["order"], 0.0)
    return model


def prune_variants(M):
    """(name, kwargs) of the prune calls each model fixture pins."""
    mask = np.ones(M, dtype=bool)
    mask[-3:] = False
    return [("default", {}), ("ridge", dict(ridge=1e-3)), ("mask", dict(mask=mask)),
            ("penalty2", dict(penalty=2.0))]


def prune_scenarios():
    """Small backward-pass problems (float64 B, as a user may pass): an exact
    fit, tiny noise columns, a zero-variance column, a masked term, a ridge, an
    intercept alone, observation weights, two nearly equal noise columns.
    Returns a list of (B, y, w or None, kwargs)."""
    rng = np.random.default_rng(31)
    out = []
    n = 200
    x = rng.standard_normal((n, 4))
    B = np.column_stack([np.ones(n), x[:, 0], x[:, 1]])
    out.append((B, B @ np.array([1.0, 3.0, -2.0]), None, dict(n_true=n)))
    B = np.column_stack([np.ones(n), x[:, 0], 0.01 * x[:, 1], 0.01 * x[:, 2]])
    out.append((B, 5.0 + 3.0 * x[:, 0], None, dict(n_true=n)))
    B = np.column_stack([np.ones(n), x[:, 0], np.zeros(n)])
    out.append((B, 2.0 + 4.0 * x[:, 0], None, {}))
    B = np.column_stack([np.ones(n), x[:, 0], x[:, 1]])
    out.append((B, 1.0 + 2.0 * x[:, 0] + 3.0 * x[:, 1], None,
                dict(mask=np.array([True, True, False]))))
    B = np.column_stack([np.ones(n), x[:, 2]])
    out.append((B, B @ np.array([5.0, 10.0]), None, dict(ridge=0.5)))
    out.append((np.ones((100, 1)), np.full(100, 3.0), None, {}))
    B = np.column_stack([np.ones(300), rng.standard_normal((300, 2))])
    out.append((B, 1.0 + 2.0 * B[:, 1] - 0.5 * B[:, 2], rng.uniform(0.1, 2.0, 300), {}))
    n = 50
    shared = 0.15 * rng.standard_normal(n)
    B = np.column_stack([np.ones(n), rng.standard_normal((n, 2)),
                         shared + 0.01 * rng.standard_normal(n),
                         shared + 0.01 * rng.standard_normal(n)])
    out.append((B, 1.0 + 2.0 * B[:, 1] - 1.5 * B[:, 2], None, {}))
    return out
