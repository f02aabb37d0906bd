"""The tensor-core projection of the mixed-precision fast pass.

mars_gpu_fast_project (use_tc=1) runs k_tc_tgemm / k_tc_project: tcgen05.mma
(kind::tf32) fed by TMA, with every FP32 operand split into two TF32 terms
and three products accumulated in FP32 in tensor memory. Its results are
compared with an FP64 restatement of the same projection on the same f32
inputs (candidate v = B[:, b] * (X[:, x] * s[x]) in f32; T = Bo^T v;
Bx = v - Bo T), and with the FP32 SIMT kernels it replaces.

Tolerances (stated per test): split TF32 keeps ~21 mantissa bits of each
product and accumulates in FP32, so an entry of T or Bx is within
TOL_REL = 2e-5 of the scale of its terms (sum |Bo| |v| for T; |v| + sum
|Bo| |T| for Bx). A single TF32 term per operand (10 bits) would miss that
by about 50x, so the bound also shows the split is in effect.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_REL = 2e-5


def _problem(n, m, p, P, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, m)))
    Bo = np.asfortranarray(Q.astype(np.float32))
    nb = m + 2
    B = rng.standard_normal((n, nb)).astype(np.float32)
    B[:, 0] = 1.0
    B[:, 1] = np.maximum(B[:, 1], 0)  # a hinge-like parent with zero stretches
    B = np.asfortranarray(B)
    X = np.asfortranarray(rng.standard_normal((n, p)).astype(np.float32))
    X[:, 2] = Bo[:, 0] * 3.0  # a candidate almost in the span of the basis
    s = (1.0 / np.sqrt((X.astype(np.float64) ** 2).mean(axis=0))).astype(np.float32)
    cand_x = np.sort(rng.integers(0, p, P)).astype(np.int32)
    cand_b = rng.integers(0, nb, P).astype(np.int32)
    cand_x[:3] = 2
    cand_b[:3] = 0
    y = rng.standard_normal(n).astype(np.float32)
    return B, X, s, cand_x, cand_b, Bo, y


def _v(B, X, s, cand_x, cand_b):
    """The candidate columns exactly as the kernels form them (f32 products)."""
    xs = (X[:, cand_x] * s[cand_x]).astype(np.float32)
    return (B[:, cand_b] * xs).astype(np.float32)


@pytest.mark.parametrize("n,m,P", [(50_000, 20, 300), (70_001, 63, 200), (4_000, 5, 1),
                                   (33_333, 128, 129)])
def test_tc_one_pass_matches_fp64(gpu, n, m, P):
    from mars_gb300 import marslib

    B, X, s, cx, cb, Bo, y = _problem(n, m, 7, P, seed=n + m)
    T, Bx, _, _ = marslib.fast_project(B, X, s, cx, cb, Bo, m, y, 1e-14, use_tc=True, passes=1)
    V = _v(B, X, s, cx, cb).astype(np.float64)
    Q = Bo.astype(np.float64)
    T_ref = V.T @ Q                            # (P, m)
    T_scale = np.abs(V).T @ np.abs(Q)
    assert np.all(np.abs(T - T_ref) <= TOL_REL * T_scale + 1e-30)
    # the projection uses the kernel's own f32 coefficients
    Tk = T.astype(np.float64)
    Bx_ref = V - Q @ Tk.T
    Bx_scale = np.abs(V) + np.abs(Q) @ np.abs(Tk).T
    assert np.all(np.abs(Bx - Bx_ref) <= TOL_REL * Bx_scale + 1e-30)


@pytest.mark.parametrize("n,m,P", [(60_000, 31, 257), (20_000, 63, 64)])
def test_tc_two_passes_against_fp64_and_simt(gpu, n, m, P):
    """Both passes, the norms and ybx: the tensor-core path stays as close to
    the exact FP64 projection as the FP32 SIMT path does."""
    from mars_gb300 import marslib

    B, X, s, cx, cb, Bo, y = _problem(n, m, 9, P, seed=7 * n + m)
    tol = 1e-14
    _, Bx_tc, s_tc, ybx_tc = marslib.fast_project(B, X, s, cx, cb, Bo, m, y, tol, use_tc=True)
    _, Bx_si, s_si, ybx_si = marslib.fast_project(B, X, s, cx, cb, Bo, m, y, tol, use_tc=False)
    V = _v(B, X, s, cx, cb).astype(np.float64)
    Q = Bo.astype(np.float64)
    # exact FP64 projection onto the complement of span(Bo) (Bo as stored in f32)
    G = Q.T @ Q
    Bx_ref = V - Q @ np.linalg.solve(G, Q.T @ V)
    vnorm = np.linalg.norm(V, axis=0)
    err_tc = np.linalg.norm(Bx_tc - Bx_ref, axis=0) / vnorm
    err_si = np.linalg.norm(Bx_si - Bx_ref, axis=0) / vnorm
    assert err_tc.max() <= 1e-6, err_tc.max()
    assert err_tc.max() <= 4.0 * err_si.max() + 1e-7
    # what is left in the span of the basis after the second pass
    inspan = np.linalg.norm(Q.T @ Bx_tc.astype(np.float64), axis=0) / vnorm
    assert inspan.max() <= 1e-6, inspan.max()
    # norms and ybx of the stored columns (FP32 per thread, FP64 across)
    s_ref = (Bx_tc.astype(np.float64) ** 2).sum(axis=0)
    np.testing.assert_allclose(s_tc, s_ref, rtol=1e-5, atol=1e-12 * vnorm.max() ** 2)
    live = s_ref > tol
    ybx_ref = (Bx_tc.astype(np.float64).T @ y.astype(np.float64)) / np.sqrt(s_ref + tol)
    np.testing.assert_allclose(ybx_tc[live], ybx_ref[live], rtol=1e-4,
                               atol=1e-5 * np.linalg.norm(y))
    # and they agree with the SIMT path's values to the same order
    np.testing.assert_allclose(s_tc, s_si, rtol=1e-4, atol=1e-10 * vnorm.max() ** 2)


def test_tc_rejects_a_basis_too_wide(gpu):
    from mars_gb300 import marslib

    B, X, s, cx, cb, Bo, y = _problem(2000, 129, 3, 4, seed=1)
    with pytest.raises(RuntimeError, match="1..128 basis columns"):
        marslib.fast_project(B, X, s, cx, cb, Bo, 129, y, 1e-14, use_tc=True, passes=1)
