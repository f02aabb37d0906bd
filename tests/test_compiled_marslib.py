"""The compiled `marslib` module (mars_gb300/pybind/marslib.cpp): the
reference's pybind11 binding (marslib.cc:152-179) rebuilt over the C ABI.

CPU: it loads, exposes the reference's class and methods, and refuses bad
layouts with the reference's messages before any device work; the
reference's own mars.py imports it as its marslib (where the reference
checkout is present). GPU: fits through it reach the reference's term paths.
"""
import os
import sys

import numpy as np
import pytest

from tests.golden import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def cmarslib(built_lib):
    from mars_gb300 import build, marslib

    if build.build_marslib() is None:
        pytest.skip("pybind11 headers not available: compiled marslib not built")
    return marslib.compiled()


def test_surface(cmarslib):
    assert cmarslib.__version__ == "0.12"
    for name in ("eval", "append", "nbasis", "yvar"):
        assert hasattr(cmarslib.MarsAlgo, name)


def test_layout_errors_before_device_work(cmarslib):
    X = np.zeros((10, 2), dtype=np.float32)  # C order: not column-major
    y = np.zeros(10, dtype=np.float32)
    with pytest.raises(RuntimeError, match="X must be column-major"):
        cmarslib.MarsAlgo(X, y, y, 5)
    Xf = np.asfortranarray(X)
    with pytest.raises(RuntimeError, match="invalid dimension for y"):
        cmarslib.MarsAlgo(Xf, y[:5], y, 5)
    with pytest.raises(TypeError):  # no implicit conversion, as the reference
        cmarslib.MarsAlgo(Xf.astype(np.float64), y, y, 5)


def test_reference_mars_py_imports_it(cmarslib, monkeypatch):
    ref = os.environ.get("MARS_REFERENCE_DIR")
    if not ref or not os.path.isfile(os.path.join(ref, "mars.py")):
        pytest.skip("reference checkout not present")
    import importlib.util

    monkeypatch.setitem(sys.modules, "marslib", cmarslib)
    spec = importlib.util.spec_from_file_location("ref_mars_over_gpu", os.path.join(ref, "mars.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    assert mod.marslib is cmarslib and mod.__version__ == "0.12"


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["plain_fit", "hinge_search_small", "weighted_nan",
                                  "fastmars_caps"])
def test_fit_through_compiled_marslib(cmarslib, gpu, name):
    from mars_gb300.mars import forward_pass
    from tests.test_oracle import assert_same_path, load_fit

    g = load_fit(name)
    X, y, w, kw = cases.fit_case(name)
    model = forward_pass(cmarslib, X, y, w, **kw)
    assert_same_path(model, g)


@pytest.mark.gpu
def test_compiled_marslib_mixed_precision(cmarslib, gpu, monkeypatch):
    from mars_gb300.mars import forward_pass
    from tests.test_oracle import assert_same_path, load_fit

    monkeypatch.setenv("MARS_GPU_PRECISION", "mixed")
    g = load_fit("hinge_search")
    X, y, w, kw = cases.fit_case("hinge_search")
    assert_same_path(forward_pass(cmarslib, X, y, w, **kw), g)
