"""Differentiable prediction (mars_gb300.diff): the CUDA expand/backward kernels
against the numpy expand (mars.py:423-450 restated in mars_gb300.mars.expand)
and FP64 central finite differences (h = 1e-6) on 1,000 rows."""
import numpy as np
import pytest

from mars_gb300 import mars
from tests.test_oracle import load_fit

pytestmark = pytest.mark.gpu


def _model(name="hinge_search_small"):
    g = load_fit(name)
    rows = g["model"]
    dt = [("type", "S1"), ("basis", "i4"), ("input", "i4"), ("hinge", "f8"), ("beta", "f4"),
          ("r2", "f4"), ("r2_cv", "f4"), ("order", "i4"), ("time", "f4")]
    model = np.zeros(len(rows), dtype=dt)
    for j, r in enumerate(rows):
        model[j]["type"] = r["type"].encode()
        model[j]["basis"] = r["basis"]
        model[j]["input"] = r["input"]
        model[j]["hinge"] = np.nan if r["hinge"] is None else r["hinge"]
    return model, g["shape"][1]


def _loss64(X, model, beta, knots, g):
    m = model.copy()
    hinge = np.isin(m["type"], (b"+", b"-"))
    m["hinge"][hinge] = knots[hinge]
    B = mars.expand(np.asfortranarray(X.astype(np.float64)), m)
    return float(g @ (B @ beta))


def _setup(seed=0, n=1000):
    import torch

    model, p = _model()
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, p)).astype(np.float32)
    M = len(model)
    beta = rng.uniform(-1, 1, M).astype(np.float64)
    knots = np.nan_to_num(model["hinge"]).astype(np.float64)
    g = rng.standard_normal(n)
    dev = torch.device("cuda", 0)
    return torch, dev, model, X, beta, knots, g


def test_predict_matches_numpy_expand(gpu):
    from mars_gb300 import diff

    torch, dev, model, X, beta, knots, g = _setup()
    Xt = torch.tensor(X, device=dev)
    pred = diff.predict(Xt, model, torch.tensor(beta, dtype=torch.float32, device=dev),
                        torch.tensor(knots, dtype=torch.float32, device=dev))
    B = mars.expand(np.asfortranarray(X.astype(np.float64)), model)
    want = B @ beta.astype(np.float32).astype(np.float64)
    np.testing.assert_allclose(pred.cpu().numpy(), want, rtol=1e-5, atol=1e-5)


def test_gradients_match_fp64_central_differences(gpu):
    from mars_gb300 import diff

    torch, dev, model, X, beta, knots, g = _setup(seed=1)
    beta32 = beta.astype(np.float32)
    knots32 = knots.astype(np.float32)
    Xt = torch.tensor(X, device=dev, requires_grad=True)
    bt = torch.tensor(beta32, device=dev, requires_grad=True)
    kt = torch.tensor(knots32, device=dev, requires_grad=True)
    pred = diff.predict(Xt, model, bt, kt)
    (pred.double() * torch.tensor(g, device=dev)).sum().backward()
    h = 1e-6
    b64, k64 = beta32.astype(np.float64), knots32.astype(np.float64)
    # beta: exactly linear
    fd_b = np.array([(_loss64(X, model, b64 + h * e, k64, g) - _loss64(X, model, b64 - h * e, k64, g))
                     / (2 * h) for e in np.eye(len(b64))])
    np.testing.assert_allclose(bt.grad.cpu().numpy(), fd_b, rtol=2e-4, atol=1e-3)
    # knots of the hinge terms
    hinge = np.where(np.isin(model["type"], (b"+", b"-")))[0]
    assert len(hinge) > 0
    for j in hinge:
        e = np.zeros_like(k64)
        e[j] = h
        fd = (_loss64(X, model, b64, k64 + e, g) - _loss64(X, model, b64, k64 - e, g)) / (2 * h)
        assert kt.grad[j].item() == pytest.approx(fd, rel=2e-4, abs=1e-3)
    # X, a sample of entries on columns the model uses
    cols = sorted(set(int(c) for c in model["input"][1:]))
    rng = np.random.default_rng(7)
    for _ in range(20):
        i, c = int(rng.integers(len(X))), int(rng.choice(cols))
        Xp, Xm = X.astype(np.float64).copy(), X.astype(np.float64).copy()
        Xp[i, c] += h
        Xm[i, c] -= h
        fd = (_loss64(Xp, model, b64, k64, g) - _loss64(Xm, model, b64, k64, g)) / (2 * h)
        assert Xt.grad[i, c].item() == pytest.approx(fd, rel=2e-4, abs=1e-4)


def test_refine_knots_reduces_rss(gpu):
    from mars_gb300 import diff, workloads

    import torch

    X, y, kw = workloads.hinge_search(n=20_000, p=6, seed=2, max_terms=9)
    model = mars.fit(X, y, **kw)
    dev = torch.device("cuda", 0)
    Xt = torch.tensor(np.asarray(X), device=dev)
    yt = torch.tensor(y, device=dev)
    # start from knots moved off the fitted ones
    m2 = model.copy()
    hinge = np.isin(m2["type"], (b"+", b"-"))
    m2["hinge"][hinge] += 0.05
    knots, beta, hist = diff.refine_knots(Xt, yt, m2, steps=200, lr=2e-3)
    assert len(hist) == 200
    assert hist[-1] < hist[0]
