"""The reference's unit-test scenarios, restated over an interchangeable backend.

Each function takes a backend (the CPU oracle or the GPU library) and asserts
the reference's structural facts with the reference's tolerances:

  delta_sse        tests/unittest.cc:213-399   (eval/append vs least squares)
  weighted_ls      tests/unittest.cc:408-448
  min_span         tests/unittest.cc:460-503
  orthonormalize   tests/test_kernels.cc:120-174, 256-353, 369-525
  orthonormalize_col  tests/test_kernels.cc:576-662

Eigen's Random() (uniform on [-1, 1]) is replaced by seeded numpy draws of the
same distribution; the reference's own inputs are not reproducible without
Eigen, so the tolerances and structural assertions are the pinned contract.
"""
import numpy as np


class OracleBackend:
    """CPU oracle (the C restatement)."""

    name = "port"

    def __init__(self, kind="port"):
        import oracle

        self.kind = kind
        self.L = oracle.load(kind)
        self._oracle = oracle

    def algo(self, X, y, w, max_terms):
        return self._oracle.OracleAlgo(X, y, w, max_terms, kind=self.kind)

    def orthonormalize(self, B, x, mask, Bo, m, tol):
        Bx, T, s, dgks = self.L.k_orthonormalize(B, x, mask, Bo, m, tol)
        return Bx, s, dgks

    def orthonormalize_col(self, v, Bo, m, tol):
        return self.L.k_orthonormalize_col(v, Bo, m, tol)


class GpuBackend:
    """The GB300 library through its C ABI."""

    name = "gpu"

    def __init__(self, precision=None):
        from mars_gb300 import marslib

        self.marslib = marslib
        self.precision = precision

    def algo(self, X, y, w, max_terms):
        a = self.marslib.MarsAlgo(X, y, w, max_terms)
        if self.precision:
            a.set_precision(self.precision)
        return a

    def orthonormalize(self, B, x, mask, Bo, m, tol):
        return self.marslib.orthonormalize(B, x, mask, Bo, m, tol)

    def orthonormalize_col(self, v, Bo, m, tol):
        return self.marslib.orthonormalize_col(v, Bo, m, tol)


def eval_col(algo, xcol, p, mask_row, min_span=1, end_span=0, linear=False):
    """Evaluate one candidate column (the reference's per-column eval())."""
    m = algo.nbasis()
    mask = np.zeros((p, m), dtype=bool)
    mask[xcol, :] = np.asarray(mask_row, dtype=bool)[:m]
    d, lin, hin, cut = algo.eval(mask, min_span, end_span, linear, 1)
    return d, lin[xcol], hin[xcol], cut[xcol]


def _slow_dsse(X, y):
    b, *_ = np.linalg.lstsq(X, y, rcond=None)
    return float(b @ (X.T @ y)) / float(y @ y)


def _slow_mse(X, y):
    b, *_ = np.linalg.lstsq(X, y, rcond=None)
    e = X @ b - y
    return float(e @ e) / len(e) / float(y @ y)


def delta_sse(be, hinge_tol, seed=0):
    """unittest.cc:213-399: eval/append agree with least squares."""
    rng = np.random.default_rng(seed)
    N, M, CUT = 5891, 13, 0.25
    X = rng.uniform(-1, 1, (N, M))
    X[100, 7] = CUT
    X[:, 10] = 0.0
    x3, x7, x9 = X[:, 3], X[:, 7], X[:, 9]
    y = (x3 * .3 - x9 * .2 + x3 * x9 * .25 - 5 * np.maximum(x7 - CUT, 0)
         + 2 * np.maximum(CUT - x7, 0))
    y = y + rng.uniform(-1, 1, N)
    X32 = np.asfortranarray(X.astype(np.float32))
    y32 = y.astype(np.float32)
    Xd = X32.astype(np.float64)
    yd = y32.astype(np.float64)
    w32 = np.ones(N, np.float32)
    algo = be.algo(X32, y32, w32, M // 2)
    ALL = np.zeros((N, 16))
    ALL[:, 0] = 1
    mask = np.zeros(M, bool)
    mask[0] = True
    nb = 1

    for xcol, bcol, newcol in [(3, 0, Xd[:, 3]), (9, 0, Xd[:, 9]),
                               (9, 1, Xd[:, 3] * Xd[:, 9])]:
        d, lin, hin, cut = eval_col(algo, xcol, M, mask[:nb], linear=True)
        if bcol:
            assert int(np.argmax(lin)) == bcol
        ALL[:, nb] = newcol
        assert abs((d + lin[bcol]) - _slow_dsse(ALL[:, :nb + 1], yd)) < 1e-7
        mse1 = algo.append("l", xcol, bcol, 0)
        mask[nb] = True
        nb += 1
        assert abs(mse1 - _slow_mse(ALL[:, :nb], yd)) < 1e-8

    # the hinge at x7 (parent = intercept) and the permutations over parents
    d, lin, hin, cut = eval_col(algo, 7, M, mask[:nb], linear=False)
    assert int(np.argmax(hin)) == 0
    assert np.all(hin[:nb] > lin[:nb])
    for b in range(nb):
        ALL[:, nb] = ALL[:, b] * np.maximum(Xd[:, 7] - cut[b], 0)
        ALL[:, nb + 1] = ALL[:, b] * np.maximum(cut[b] - Xd[:, 7], 0)
        ref = _slow_dsse(ALL[:, :nb + 2], yd)
        assert abs((d + hin[b]) / N - ref / N) < hinge_tol, (b, d + hin[b], ref)
    ALL[:, nb] = np.maximum(Xd[:, 7] - CUT, 0)
    ALL[:, nb + 1] = np.maximum(CUT - Xd[:, 7], 0)
    assert abs((d + hin[0]) / N - _slow_dsse(ALL[:, :nb + 2], yd) / N) < hinge_tol

    mse1 = algo.append("+", 7, 0, CUT)
    mask[nb] = True
    nb += 1
    assert abs(mse1 - _slow_mse(ALL[:, :nb], yd)) < 2e-8
    mse1 = algo.append("-", 7, 0, CUT)
    mask[nb] = True
    nb += 1
    assert abs(mse1 - _slow_mse(ALL[:, :nb], yd)) < 1e-7
    last_mse = mse1

    # an all-zero input column adds nothing
    d, lin, hin, cut = eval_col(algo, 10, M, mask[:nb], linear=False)
    assert abs(d - (1 - last_mse * N)) < 1e-8
    assert np.all(lin[:nb] == 0) and np.all(hin[:nb] == 0)

    # masking a parent: its outputs are zero/NaN, the others unchanged
    mask2 = mask.copy()
    mask2[3] = False
    _, l1, h1, c1 = eval_col(algo, 2, M, mask2[:nb])
    assert np.isnan(c1[3]) and l1[3] == 0 and h1[3] == 0
    _, l2, h2, c2 = eval_col(algo, 2, M, mask[:nb])
    keep = np.arange(nb) != 3
    np.testing.assert_allclose(l1[keep], l2[keep], rtol=1e-12, atol=0)
    np.testing.assert_allclose(h1[keep], h2[keep], rtol=1e-12, atol=0)
    np.testing.assert_array_equal(c1[keep], c2[keep])


def weighted_ls(be, seed=0):
    """unittest.cc:408-448: the sqrt(w) row scaling reproduces closed-form WLS."""
    rng = np.random.default_rng(seed)
    N, M = 1000, 4
    X = rng.uniform(-1, 1, (N, M))
    y = X[:, 1] * 0.5 + X[:, 2] * 0.3 + rng.uniform(-1, 1, N) * 0.1
    w = 0.01 + 10.0 * np.abs(X[:, 0])
    X32 = np.asfortranarray(X.astype(np.float32))
    y32, w32 = y.astype(np.float32), w.astype(np.float32)
    algo = be.algo(X32, y32, w32, M)
    Xd, yd, wd = X32.astype(float), y32.astype(float), w32.astype(float)

    def wls(A):
        sw = np.sqrt(wd)
        b, *_ = np.linalg.lstsq(A * sw[:, None], yd * sw, rcond=None)
        e = A @ b - yd
        return float((wd * e * e).sum()) / N / float((wd * yd * yd).sum())

    A = np.ones((N, 1))
    for col in (1, 2):
        mse = algo.append("l", col, 0, 0)
        A = np.column_stack([A, Xd[:, col]])
        assert abs(mse - wls(A)) < 1e-7


def min_span(be, seed=0):
    """unittest.cc:460-503: min_span only restricts which cuts are scored."""
    rng = np.random.default_rng(seed)
    N, M, CUT = 2000, 4, 0.25
    X = rng.uniform(-1, 1, (N, M))
    y = -5 * np.maximum(X[:, 0] - CUT, 0) + 2 * np.maximum(CUT - X[:, 0], 0)
    y = y + rng.uniform(-1, 1, N) * 0.05
    algo = be.algo(np.asfortranarray(X.astype(np.float32)), y.astype(np.float32),
                   np.ones(N, np.float32), M * 2)
    r = {s: eval_col(algo, 0, M, [True], min_span=s) for s in (1, 2, 10)}
    assert r[1][2][0] >= r[2][2][0] >= r[10][2][0]
    assert abs(r[1][1][0] - r[2][1][0]) <= 1e-12
    assert abs(r[1][1][0] - r[10][1][0]) <= 1e-12
    for s in (1, 2, 10):
        assert abs(r[s][3][0] - CUT) < 0.05


def make_orthonormal_basis(n, m, rng, bad_col=-1):
    """Orthonormal f32 basis built by modified Gram-Schmidt in f64
    (test_kernels.cc:25-50); `bad_col` duplicates its predecessor first."""
    B = rng.uniform(-1, 1, (n, m)).astype(np.float32).astype(np.float64)
    if 0 < bad_col < m:
        B[:, bad_col] = B[:, bad_col - 1]
    Q = B.copy()

    def unit(v):
        s = np.linalg.norm(v)
        return v / s if s > 1e-14 else v * 0.0

    Q[:, 0] = unit(Q[:, 0])
    for j in range(1, m):
        Q[:, j] = unit(Q[:, j])
        for k in range(j):
            Q[:, j] -= (Q[:, k] @ Q[:, j]) * Q[:, k]
            Q[:, j] = unit(Q[:, j])
    return np.ascontiguousarray(Q.astype(np.float32))


def _numpy_orthonormalize(B, x, mask, Bo, m, tol):
    Bx = (B[:, mask].astype(np.float32) * x[:, None]).astype(np.float64)
    Q = Bo[:, :m].astype(np.float64)
    Bx -= Q @ (Q.T @ Bx)
    s = (Bx * Bx).sum(axis=0)
    scale = np.where(s > tol, 1 / np.sqrt(s + tol), 0.0)
    return Bx * scale


def orthonormalize_basic(be, seed=0):
    """test_kernels.cc:120-174 and 256-353."""
    rng = np.random.default_rng(seed)
    n, m, p, tol = 89, 13, 7, 1e-14
    Bo = make_orthonormal_basis(n, m, rng)
    B = rng.uniform(-1, 1, (n, m)).astype(np.float32)
    x = rng.uniform(-1, 1, n).astype(np.float32)
    mask = np.sort(rng.permutation(m)[:p]).astype(np.int32)
    Bx, s, dgks = be.orthonormalize(np.asfortranarray(B), x, mask, Bo, m, tol)
    Q = Bo.astype(np.float64)
    Bxd = Bx.astype(np.float64)
    assert np.abs(Q.T @ Q - np.eye(m)).max() < 1e-5
    assert np.abs(Q.T @ Bxd).max() < 1e-5
    assert np.abs(np.linalg.norm(Bxd, axis=0) - 1).max() < 1e-5
    assert np.abs(Bxd - _numpy_orthonormalize(B, x, mask, Bo, m, tol)).max() < 1e-5

    # DGKS fires exactly once on a 95%/5% split (test_kernels.cc:256-318)
    n, m = 200, 4
    Bo = make_orthonormal_basis(n, m, rng)
    Q = Bo.astype(np.float64)
    v = rng.uniform(-1, 1, n)
    v -= Q @ (Q.T @ v)
    v /= np.linalg.norm(v)
    B = np.zeros((n, m), np.float32)
    B[:, 0] = (np.sqrt(0.95) * Q[:, 0] + np.sqrt(0.05) * v).astype(np.float32)
    Bx, s, dgks = be.orthonormalize(np.asfortranarray(B), np.ones(n, np.float32),
                                    np.array([0], np.int32), Bo, m, 1e-14)
    assert dgks == 1
    assert np.abs(Q.T @ Bx.astype(np.float64)).max() < 1e-5
    assert abs(np.linalg.norm(Bx[:, 0].astype(np.float64)) - 1) < 1e-5

    # ... and never on well-conditioned columns (test_kernels.cc:320-353)
    n, m, p = 89, 4, 3
    Bo = make_orthonormal_basis(n, m, rng)
    B = rng.uniform(-1, 1, (n, p)).astype(np.float32)
    _, _, dgks = be.orthonormalize(np.asfortranarray(B), np.ones(n, np.float32),
                                   np.arange(p, dtype=np.int32), Bo, m, 1e-14)
    assert dgks == 0


def orthonormalize_stress(be, seed=0):
    """test_kernels.cc:369-525: mixed magnitudes, a near-collinear (DGKS)
    column and an exactly degenerate one."""
    rng = np.random.default_rng(seed)
    n, m, p, tol = 8192, 128, 32, 1e-14
    Bo = make_orthonormal_basis(n, m, rng)
    Q = Bo.astype(np.float64)
    B = rng.uniform(-1, 1, (n, m)).astype(np.float32)
    B *= (2.0 ** (np.arange(m) % 5)).astype(np.float32)
    DGKS_COL, DEGEN_COL = 3, 7
    v = rng.uniform(-1, 1, n)
    v -= Q @ (Q.T @ v)
    v /= np.linalg.norm(v)
    B[:, DGKS_COL] = (np.sqrt(0.97) * Q[:, 0] + np.sqrt(0.03) * v).astype(np.float32)
    B[:, DEGEN_COL] = Bo[:, 1]
    rest = [j for j in range(m) if j not in (DGKS_COL, DEGEN_COL)]
    rng.shuffle(rest)
    mask = np.sort(np.array([DGKS_COL, DEGEN_COL] + rest[:p - 2], dtype=np.int32))
    dj = int(np.where(mask == DGKS_COL)[0][0])
    gj = int(np.where(mask == DEGEN_COL)[0][0])
    x = np.ones(n, np.float32)
    Bx, s, dgks = be.orthonormalize(np.asfortranarray(B), x, mask, Bo, m, tol)
    Bxd = Bx.astype(np.float64)
    assert dgks >= 1
    assert np.abs(Q.T @ Bxd).max() < 1e-6
    for j in range(p):
        if j != gj:
            assert abs((Bxd[:, j] ** 2).sum() - 1) < 1e-5
    assert float((Bx[:, gj] ** 2).sum()) == 0.0
    ref = _numpy_orthonormalize(B, x, mask, Bo, m, tol)
    for j in range(p):
        if j not in (dj, gj):
            assert np.abs(Bxd[:, j] - ref[:, j]).max() < 1e-5
    return Bx, s, dgks


def orthonormalize_col_cases(be, seed=0):
    """test_kernels.cc:576-662."""
    rng = np.random.default_rng(seed)
    n, m = 89, 13
    Bo = make_orthonormal_basis(n, m, rng)
    Q = Bo.astype(np.float64)
    v0 = rng.uniform(-1, 1, n)
    w, v, dgks = be.orthonormalize_col(v0, Bo, m, 1e-14)
    ref = v0.copy()
    for j in range(m):
        ref -= (Q[:, j] @ ref) * Q[:, j]
    w_ref = np.linalg.norm(ref)
    assert abs(w - w_ref) <= 1e-9 * (1 + abs(w_ref))
    np.testing.assert_allclose(v, ref / w_ref, rtol=0, atol=1e-9)
    assert np.abs(Q.T @ v).max() < 1e-6
    assert dgks == 0

    n, m = 200, 4
    Bo = make_orthonormal_basis(n, m, rng)
    Q = Bo.astype(np.float64)
    u = rng.uniform(-1, 1, n)
    u -= Q @ (Q.T @ u)
    u /= np.linalg.norm(u)
    v0 = np.sqrt(0.95) * Q[:, 0] + np.sqrt(0.05) * u
    w, v, dgks = be.orthonormalize_col(v0, Bo, m, 1e-14)
    assert dgks == 1 and w > 0
    assert np.abs(Q.T @ v).max() < 1e-6
    assert abs(np.linalg.norm(v) - 1) < 1e-6

    n, m = 64, 5
    Bo = make_orthonormal_basis(n, m, rng)
    v0 = Bo[:, 2].astype(np.float64) * 1.0
    w, v, dgks = be.orthonormalize_col(v0, Bo, m, 1e-6)
    assert w * w <= 1e-6
    assert np.linalg.norm(v) < 1e-3
    assert dgks == 0
