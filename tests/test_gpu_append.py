"""The append on the GPU (mars_gb300/csrc/xappend.cu) against the oracle, bit for bit.

Every FP64 chain of MarsAlgo::append (marsalgo.cc:760-875) and of
orthonormalize_col (kernels.cc:239-281) -- the raw norm, the modified
Gram-Schmidt dots, the norm of the result, y . the new column -- runs as an
exact parallel evaluation of the reference's sequential chain: chunk records,
composed by sub-group, warp and block, walked by the last block with descents
wherever a record cannot vouch for its entry. The results must equal the
oracle's: w and v of orthonormalize_col, the MSE of every append (and its
rejection), dsse, and the eval outputs after the appends -- whose DGKS
re-pass runs on the same exact chains, side by side -- from a handful of rows
(one partly empty block) to 10^6 rows (hundreds of blocks).
"""
import numpy as np
import pytest

import oracle
from tests import scenarios

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.asarray(a, np.float64).view(np.uint64)


def _basis(n, m, rng):
    if m == 0:
        return np.zeros((n, 1), np.float32)
    if n * m <= 200_000:
        return scenarios.make_orthonormal_basis(n, m, rng)
    q, _ = np.linalg.qr(rng.standard_normal((n, m)))
    return q.astype(np.float32)


@pytest.mark.parametrize("n,m", [(1, 0), (3, 1), (7, 3), (1000, 5), (4099, 17), (65536, 8),
                                 (300_001, 30), (1_000_000, 12)])
def test_orthonormalize_col_bit_exact(gpu, port, n, m):
    rng = np.random.default_rng(n + 17 * m)
    Bo = _basis(n, m, rng)
    vs = {"random": rng.uniform(-1, 1, n),
          "signed small": rng.standard_normal(n) * 1e-3}
    if m:
        # mostly in the span: the DGKS re-pass fires
        vs["near span"] = Bo[:, 0].astype(np.float64) + 1e-3 * rng.standard_normal(n)
        # in the span: the norm falls below tol
        vs["in span"] = Bo[:, m - 1].astype(np.float64)
    for name, v0 in vs.items():
        for tol in (1e-14, 1e-6):
            wg, vg, dg = gpu.orthonormalize_col(v0, Bo, m, tol)
            wc, vc, dc = port.k_orthonormalize_col(v0, Bo, m, tol)
            assert _bits(wg) == _bits(wc), (name, tol, wg, wc)
            np.testing.assert_array_equal(_bits(vg), _bits(vc), err_msg=name)
            assert dg == dc, (name, tol)


def _problem(n, p, seed):
    r = np.random.default_rng(seed)
    X = r.standard_normal((n, p)).astype(np.float32)
    X[:, 1] = X[:, 0] + np.float32(1e-4) * r.standard_normal(n).astype(np.float32)
    y = (2 * X[:, 0] - np.maximum(X[:, 2] - 0.3, 0) + X[:, 0] * X[:, 3]
         + r.standard_normal(n)).astype(np.float32)
    w = (0.5 + r.random(n)).astype(np.float32)
    return np.asfortranarray(X), y, w


def _appends(X):
    q = lambda j, f: float(np.quantile(X[:, j], f))
    return [("l", 0, 0, float("nan")),
            ("+", 2, 0, q(2, 0.6)), ("-", 2, 0, q(2, 0.6)),
            ("l", 1, 0, float("nan")),        # nearly the column of input 0: DGKS
            ("+", 2, 0, q(2, 0.6)),           # a duplicate: rejected
            ("l", 3, 1, float("nan")),
            ("+", 0, 2, q(0, 0.3)), ("-", 1, 2, q(1, 0.3)),
            ("+", 3, 5, q(3, 0.9)), ("l", 4 % X.shape[1], 3, float("nan")),
            ("-", 0, 6, q(0, 0.95))]


@pytest.mark.parametrize("n,p,seed", [(9, 5, 0), (5000, 6, 1), (200_003, 7, 2),
                                      (1_000_000, 5, 3)])
def test_append_sequence_bit_exact(gpu, n, p, seed):
    X, y, w = _problem(n, p, seed)
    mt = 16
    g = gpu.MarsAlgo(X, y, w, mt)
    c = oracle.OracleAlgo(X, y, w, mt, kind="port")
    for k, (t, xc, bc, h) in enumerate(_appends(X)):
        if bc >= c.nbasis():
            continue
        mg = g.append(t, xc, bc, h)
        mc = c.append(t, xc, bc, h)
        assert _bits(mg) == _bits(mc), (k, t, xc, bc, mg, mc)
        assert g.nbasis() == c.nbasis(), k
    assert _bits(g.dsse()) == _bits(c.dsse())
    mask = np.ones((p, g.nbasis()), bool)
    fired = g.stats()["dgks_fired"]
    out_g = g.eval(mask, 1, 0, False, 1)
    out_c = c.eval(mask, 1, 0, False, 0)
    for a, b in zip(out_g[1:], out_c[1:]):
        np.testing.assert_array_equal(a, b)
    if n >= 65536:
        # the eval's DGKS re-pass (near-duplicate inputs 0 and 1) formed T with
        # the side-by-side exact chains (few entries, long columns)
        assert g.stats()["dgks_fired"] > fired
