"""The drop-in boundary, checked without a GPU.

* libmars_gpu.so loads and exports exactly the entry points that
  include/mars_gpu.h declares (no compute call is made);
* with no visible device, the product fails loudly (no CPU fallback);
* the Python surface keeps the reference's argument handling and the
  model/expand/pprint formats (mars.py:60-214, 423-450, 741-775).
"""
import ctypes
import io
import os
import re
import subprocess
import contextlib

import numpy as np
import pytest

from mars_gb300 import mars

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mars_gpu.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"MARS_GPU_API\s+[\w\s\*]*?\b(mars_gpu_\w+)\s*\(", text)))


def test_header_declares_the_abi():
    syms = declared_symbols()
    for name in ("mars_gpu_create", "mars_gpu_eval", "mars_gpu_append", "mars_gpu_destroy",
                 "mars_gpu_last_error", "mars_gpu_orthonormalize"):
        assert name in syms


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True,
                         text=True, check=True).stdout
    exported = sorted(set(re.findall(r"\bT (mars_gpu_\w+)", out)))
    assert exported == declared_symbols()
    lib = ctypes.CDLL(built_lib)
    for name in declared_symbols():
        assert hasattr(lib, name)


def test_no_device_fails_loudly(built_lib):
    from mars_gb300 import marslib

    marslib.load()
    if marslib.device_count() > 0:
        pytest.skip("a GPU is visible here")
    X = np.asfortranarray(np.random.default_rng(0).standard_normal((50, 2)).astype("f"))
    y = X[:, 0].copy()
    with pytest.raises(RuntimeError, match="no CUDA device"):
        marslib.MarsAlgo(X, y, np.ones(50, "f"), 5)
    with pytest.raises(RuntimeError, match="no CUDA device"):
        mars.fit(X, y, max_terms=5)


def test_layout_checks(built_lib):
    from mars_gb300 import marslib

    y = np.ones(10, "f")
    with pytest.raises(RuntimeError, match="X must be column-major"):
        marslib.MarsAlgo(np.ones((10, 3), "f"), y, y, 4)
    with pytest.raises(RuntimeError, match="expected 2D array for X"):
        marslib.MarsAlgo(np.ones(10, "f"), y, y, 4)
    with pytest.raises(RuntimeError, match="invalid dimension for y"):
        marslib.MarsAlgo(np.ones((10, 3), "f", order="F"), np.ones(9, "f"), y, 4)
    with pytest.raises(TypeError):
        marslib.MarsAlgo(np.ones((10, 3), order="F"), y, y, 4)


def test_fit_argument_checks():
    X = np.asfortranarray(np.ones((20, 2), "f"))
    with pytest.raises(TypeError, match="unknown argument"):
        mars.fit(X, np.ones(20, "f"), bogus=1)
    with pytest.raises(AssertionError, match="column-major"):
        mars.fit(np.ones((20, 2), "f"), np.ones(20, "f"))
    with pytest.raises(AssertionError, match="32-bit float"):
        mars.fit(np.ones((20, 2)), np.ones(20, "f"))
    with pytest.raises(AssertionError, match="length mismatch"):
        mars.fit(X, np.ones(19, "f"))


def _model(rows, beta):
    model = np.zeros(len(rows), dtype=mars.MODEL_DTYPE)
    for i, (t, b, x, h) in enumerate(rows):
        model[i] = (t, b, x, h, beta[i], 0, 0, 0, 0)
    return model


def test_expand_semantics():
    rng = np.random.default_rng(7)
    X = rng.standard_normal((50, 3)).astype("f")
    model = _model([("i", 0, 0, np.nan), ("l", 0, 0, np.nan), ("l", 0, 1, np.nan),
                    ("+", 1, 2, 0.5), ("-", 3, 1, -0.25)], [2.0, 3.0, 0.0, -1.0, 0.5])
    B = mars.expand(X, model)
    assert B.dtype == np.float32 and B.flags.f_contiguous and B.shape == (50, 5)
    x = X.astype(np.float32)
    np.testing.assert_array_equal(B[:, 0], 1)
    np.testing.assert_array_equal(B[:, 1], x[:, 0])
    np.testing.assert_array_equal(B[:, 2], x[:, 1])
    np.testing.assert_array_equal(B[:, 3], x[:, 0] * np.maximum(x[:, 2] - 0.5, 0))
    np.testing.assert_array_equal(B[:, 4], B[:, 3] * np.maximum(-0.25 - x[:, 1], 0))


def test_pprint_format():
    model = _model([("i", 0, 0, np.nan), ("l", 0, 0, np.nan), ("+", 1, 2, 0.5)],
                   [2.0, 3.0, -1.0])
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        mars.pprint(model, labels=["a", "b", "c"])
    lines = buf.getvalue().splitlines()
    assert lines[0] == "         +2"
    assert lines[1] == "         +3 * a"
    assert lines[2] == "         -1 * MAX(c-0.5,0) * a"
