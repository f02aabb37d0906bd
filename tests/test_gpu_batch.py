"""Concurrent independent fits (mars_gb300.batch.fit_many): every fit, driven
from its own host thread and stream, keeps the reference's term path."""
import pytest

from mars_gb300 import workloads
from tests.golden import cases
from tests.test_oracle import assert_same_path, load_fit

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fit_many_keeps_each_term_path(gpu, precision):
    from mars_gb300 import batch

    names = [n for n in cases.FIT_CASES if n.startswith("batched_small_")]
    fits = workloads.batched_fits(count=3, seed=4, n_hi=20_000, p_hi=12)
    probs = [(X, y, None, kw) for X, y, kw in fits]
    models, times = batch.fit_many(probs, threads=3, precision=precision)
    assert len(models) == 3 and all(t > 0 for t in times)
    for name, model in zip(names, models):
        assert_same_path(model, load_fit(name))
