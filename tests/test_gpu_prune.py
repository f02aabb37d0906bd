"""The backward pass on the GPU: mars.gram (mars_gpu_gram) and mars.prune.

gram is compared with a numpy restatement of the reference's arithmetic
(mars.py:456-490 over numpy's BLAS): per 128-row chunk a fused multiply-add
chain in the input dtype over the rows in order, the chunk results added in
float64 in chunk order. The restatement forms each f32 FMA as an FP64 sum
rounded to f32 (exact unless the sum needs more than 53 bits, which these
inputs never do), so the bound is 1e-15 relative. prune is compared with the
reference's own prune on the golden fits and scenarios: the same selected
terms, coefficients within 1e-5 of the largest (the reference computes its
matrix-vector Gram products with several partial sums of its BLAS build,
which cannot be followed; those run here exactly in FP64, ~1e-8 from the
reference's, and move the coefficients by ~1e-6).
"""
import json
import os

import numpy as np
import pytest

from tests.golden import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _chunk_fma_gram(A, B, dt):
    n = A.shape[0]
    total = np.zeros((A.shape[1], B.shape[1]))
    for c0 in range(0, n, 128):
        a = A[c0:c0 + 128].astype(np.float64)
        b = B[c0:c0 + 128].astype(np.float64)
        acc = np.zeros(total.shape, dtype=dt)
        for r in range(a.shape[0]):
            acc = (acc.astype(np.float64) + np.outer(a[r], b[r])).astype(dt)
        total = total + acc.astype(np.float64)
    return total


def test_gram_follows_the_reference_chunk_arithmetic(gpu):
    from mars_gb300 import mars

    rng = np.random.default_rng(3)
    A = rng.standard_normal((1000, 7)).astype(np.float32)
    B = np.abs(rng.standard_normal((1000, 19))).astype(np.float32)
    got = mars.gram(A, B)
    np.testing.assert_allclose(got, _chunk_fma_gram(A, B, np.float32), rtol=1e-15, atol=0)
    # f32 chains over 128-row chunks: within ~1e-5 of the exact FP64 product
    np.testing.assert_allclose(mars.gram(A), A.T.astype(np.float64) @ A, rtol=1e-5)


def test_gram_shapes_and_accumulation(gpu):
    """The reference's gram semantics (tests/test_prune.py there): 1-D
    arguments are columns; float64 accumulation beats a float32 sum."""
    from mars_gb300 import mars

    rng = np.random.default_rng(1)
    A = rng.standard_normal((300, 4)).astype(np.float32)
    y = rng.standard_normal(300).astype(np.float32)
    assert mars.gram(A, y).shape == (4,)
    assert mars.gram(y, A).shape == (4,)
    assert isinstance(mars.gram(y, y), float)
    # a product with a vector is exact: FP64 chains of exactly widened products
    np.testing.assert_allclose(mars.gram(A, y), A.T.astype(np.float64) @ y, rtol=1e-13)
    half = np.full((100_000, 1), 0.5, dtype=np.float32)
    assert mars.gram(half)[0, 0] == 25_000.0
    D = rng.standard_normal((500, 3))
    np.testing.assert_allclose(mars.gram(D), _chunk_fma_gram(D, D, np.float64), rtol=1e-14)
    with pytest.raises(ValueError, match="not aligned"):
        mars.gram(A, y[:10])


@pytest.mark.parametrize("fit", cases.PRUNE_MODEL_CASES)
def test_prune_matches_reference(gpu, fit):
    from mars_gb300 import mars

    ref = np.load(os.path.join(GOLDEN, "prune_%s.npz" % fit))
    rows = json.load(open(os.path.join(GOLDEN, fit + ".json")))["model"]
    X, y, w, _ = cases.fit_case(fit)
    model = cases.model_from_rows(rows)
    B = mars.expand(X, model)
    for tag, kw in cases.prune_variants(len(model)):
        beta = mars.prune(B, y, w, **kw)
        want = ref["beta_" + tag]
        np.testing.assert_array_equal(beta != 0, want != 0, err_msg=tag)
        np.testing.assert_allclose(beta, want, rtol=0, atol=1e-5 * np.abs(want).max(),
                                   err_msg=tag)


def test_prune_scenarios_match_reference(gpu):
    from mars_gb300 import mars

    ref = np.load(os.path.join(GOLDEN, "prune_scenarios.npz"))
    for i, (B, y, w, kw) in enumerate(cases.prune_scenarios()):
        beta = mars.prune(B, y, w, **kw)
        want = ref["beta_%d" % i]
        np.testing.assert_array_equal(beta != 0, want != 0, err_msg=str(i))
        np.testing.assert_allclose(beta, want, rtol=1e-9, atol=1e-9, err_msg=str(i))


def test_fit_prune_compact_pipeline(gpu):
    """fit on the GPU, prune, store beta on the model, compact: the compacted
    model predicts what the full one does."""
    from mars_gb300 import mars, workloads

    X, y, kw = workloads.hinge_search(n=20_000, p=8, seed=3, max_terms=15)
    model = mars.fit(X, y, **kw)
    model["beta"] = mars.prune(mars.expand(X, model), y)
    small = mars.compact(model)
    assert 1 <= len(small) <= len(model)
    np.testing.assert_allclose(mars.expand(X, small) @ small["beta"],
                               mars.expand(X, model) @ model["beta"], rtol=1e-5, atol=1e-4)
    back = mars.loads(mars.dumps(small))
    assert back.tobytes() == small.tobytes()
