"""ctypes wrappers over the oracle libraries (test infrastructure only).

``OracleAlgo`` mirrors the surface of the reference ``marslib.MarsAlgo``
(marslib.cc:152-179): ``eval``, ``append``, ``nbasis``, ``yvar``. The fit loop
in ``mars_gb300.mars`` can drive it through ``marslib_for(kind)`` so the
oracle's term path comes from the same orchestration code as the GPU's.
"""
import ctypes
import os
import subprocess
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout, when one is present: named by MARS_REFERENCE_DIR
# (no default; without it only the port is built).
REF_DIR = os.environ.get("MARS_REFERENCE_DIR")

_PATHS = {
    "port": os.path.join(HERE, "_build", "libmars_oracle.so"),
    "ref": os.path.join(HERE, "_ref", "libmars_ref.so"),
    "ref_scalar": os.path.join(HERE, "_ref", "libmars_ref_scalar.so"),
}
_PREFIX = {"port": "mo_", "ref": "mr_", "ref_scalar": "mr_"}
_LIBS = {}

_c_float_p = ctypes.POINTER(ctypes.c_float)
_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_long_p = ctypes.POINTER(ctypes.c_long)
_c_bool_p = ctypes.POINTER(ctypes.c_bool)
_c_i32_p = ctypes.POINTER(ctypes.c_int32)


def build(with_reference=None, quiet=True):
    """Compile the port (always) and the reference build (when its sources exist)."""
    targets = ["port"]
    ref_dir = os.environ.get("MARS_REFERENCE_DIR") or REF_DIR
    if with_reference is None:
        with_reference = bool(ref_dir) and os.path.isfile(os.path.join(ref_dir, "marsalgo.cc"))
    if with_reference:
        if not ref_dir:
            raise RuntimeError("MARS_REFERENCE_DIR must name the reference checkout")
        targets.append("ref")
    cmd = ["make", "-C", HERE, "PYTHON=" + (os.environ.get("PYTHON") or "python3")]
    if ref_dir:
        cmd.append("REF=" + ref_dir)
    out = subprocess.run(cmd + targets, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def available(kind):
    return os.path.isfile(_PATHS[kind])


def _ptr(a, t):
    return a.ctypes.data_as(t)


class OracleLib:
    """One loaded oracle library with its C API bound."""

    def __init__(self, kind):
        path = _PATHS[kind]
        if not os.path.isfile(path):
            raise RuntimeError("oracle library %r not built: %s" % (kind, path))
        self.kind = kind
        self.lib = ctypes.CDLL(path)
        p = _PREFIX[kind]
        L = self.lib

        def fn(name, res, args):
            f = getattr(L, p + name)
            f.restype = res
            f.argtypes = args
            setattr(self, name, f)

        sz = ctypes.c_size_t
        fn("create", ctypes.c_void_p,
           [_c_float_p, _c_float_p, _c_float_p, sz, sz, sz, sz, ctypes.c_char_p, sz])
        fn("destroy", None, [ctypes.c_void_p])
        fn("nbasis", ctypes.c_int, [ctypes.c_void_p])
        fn("nrows", ctypes.c_int, [ctypes.c_void_p])
        fn("yvar", ctypes.c_double, [ctypes.c_void_p])
        fn("dsse", ctypes.c_double, [ctypes.c_void_p])
        fn("eval_all", ctypes.c_int,
           [ctypes.c_void_p, _c_double_p, _c_double_p, _c_double_p, _c_bool_p,
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            ctypes.c_int, _c_long_p, ctypes.c_char_p, sz])
        fn("append", ctypes.c_double,
           [ctypes.c_void_p, ctypes.c_char, ctypes.c_int, ctypes.c_int, ctypes.c_float,
            _c_int_p, ctypes.c_char_p, sz])
        fn("argsort", None, [_c_i32_p, _c_float_p, sz])
        fn("covariates", None,
           [_c_double_p, _c_double_p, _c_float_p, _c_double_p, ctypes.c_double,
            ctypes.c_double, ctypes.c_double, ctypes.c_float, sz, _c_double_p, _c_double_p])
        fn("orthonormalize", None,
           [sz, sz, sz, _c_float_p, sz, _c_float_p, _c_int_p, _c_float_p, sz,
            _c_float_p, sz, _c_double_p, sz, _c_double_p, ctypes.c_double, _c_long_p])
        fn("orthonormalize_col", ctypes.c_double,
           [sz, sz, _c_double_p, _c_float_p, sz, ctypes.c_double, _c_long_p])
        fn("dot_widen", ctypes.c_double, [_c_float_p, _c_float_p, sz])
        if kind == "port":
            fn("tol", ctypes.c_double, [ctypes.c_void_p])
            fn("get_state", None,
               [ctypes.c_void_p, _c_float_p, _c_float_p, _c_float_p, _c_double_p, _c_float_p])

    # -- kernel-level helpers (used by the kernel tests) -----------------------
    def k_argsort(self, v):
        v = np.ascontiguousarray(v, dtype=np.float32)
        k = np.empty(len(v), dtype=np.int32)
        self.argsort(_ptr(k, _c_i32_p), _ptr(v, _c_float_p), len(v))
        return k

    def k_orthonormalize(self, B, x, mask, Bo, m, tol):
        """B (n, *) col-major f32; Bo (n, >=m) row-major f32. Returns (Bx, T, s, dgks)."""
        B = np.asfortranarray(B, dtype=np.float32)
        Bo = np.ascontiguousarray(Bo, dtype=np.float32)
        x = np.ascontiguousarray(x, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.int32)
        n, p = B.shape[0], len(mask)
        Bx = np.zeros((n, p), dtype=np.float32, order="F")
        T = np.zeros((max(m, 1), p), dtype=np.float64, order="F")
        s = np.zeros(p, dtype=np.float64)
        c = ctypes.c_long(0)
        self.orthonormalize(n, m, p, _ptr(B, _c_float_p), n, _ptr(x, _c_float_p),
                            _ptr(mask, _c_int_p), _ptr(Bo, _c_float_p), Bo.shape[1],
                            _ptr(Bx, _c_float_p), n, _ptr(T, _c_double_p), max(m, 1),
                            _ptr(s, _c_double_p), tol, ctypes.byref(c))
        return Bx, T, s, c.value

    def k_orthonormalize_col(self, v, Bo, m, tol):
        v = np.array(v, dtype=np.float64)
        Bo = np.ascontiguousarray(Bo, dtype=np.float32)
        c = ctypes.c_long(0)
        w = self.orthonormalize_col(len(v), m, _ptr(v, _c_double_p), _ptr(Bo, _c_float_p),
                                    Bo.shape[1], tol, ctypes.byref(c))
        return w, v, c.value


class OracleAlgo:
    """marslib.MarsAlgo-compatible object backed by an oracle library."""

    def __init__(self, X, y, w, max_terms, kind="port"):
        self._L = load(kind)
        X = np.asarray(X)
        y = np.asarray(y)
        w = np.asarray(w)
        if X.ndim != 2:
            raise RuntimeError("expected 2D array for X")
        if y.ndim != 1:
            raise RuntimeError("expected 1D array for y")
        if w.ndim != 1:
            raise RuntimeError("expected 1D array for w")
        if X.dtype != np.float32 or X.strides[0] != 4:
            raise RuntimeError("X must be column-major")
        if y.dtype != np.float32 or y.strides[0] != 4:
            raise RuntimeError("y must be column-major")
        if w.dtype != np.float32 or w.strides[0] != 4:
            raise RuntimeError("w must be column-major")
        if X.shape[0] != y.shape[0]:
            raise RuntimeError("invalid dimension for y")
        if X.shape[0] != w.shape[0]:
            raise RuntimeError("invalid dimension for w")
        self._X = X  # borrowed, like keep_alive<1,2>
        ldx = X.strides[1] // 4 if X.shape[1] > 1 else X.shape[0]
        err = ctypes.create_string_buffer(256)
        h = self._L.create(_ptr(X, _c_float_p), _ptr(y, _c_float_p), _ptr(w, _c_float_p),
                           X.shape[0], X.shape[1], int(max_terms), ldx, err, 256)
        if not h:
            raise RuntimeError(err.value.decode())
        self._h = h
        self.dgks_count = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.destroy(h)
            self._h = None

    def nbasis(self):
        return self._L.nbasis(self._h)

    def yvar(self):
        return self._L.yvar(self._h)

    def dsse(self):
        return self._L.dsse(self._h)

    def eval(self, mask, min_span, endspan, linear_only, threads, cuda=False):
        if mask.ndim != 2:
            raise RuntimeError("expected 2D array for mask")
        if mask.dtype != np.bool_ or mask.strides[1] != 1:
            raise RuntimeError("mask must be row-major")
        m = self.nbasis()
        if mask.shape[1] != m:
            raise RuntimeError("invalid dimension for mask")
        if min_span < 1:
            raise RuntimeError("min_span must be >= 1")
        rows = mask.shape[0]
        lin = np.empty((rows, m))
        hin = np.empty((rows, m))
        cut = np.empty((rows, m))
        err = ctypes.create_string_buffer(256)
        c = ctypes.c_long(0)
        rc = self._L.eval_all(self._h, _ptr(lin, _c_double_p), _ptr(hin, _c_double_p),
                              _ptr(cut, _c_double_p), _ptr(mask, _c_bool_p), rows,
                              mask.strides[0], int(min_span), int(endspan),
                              int(bool(linear_only)), int(threads), ctypes.byref(c), err, 256)
        if rc != 0:
            raise RuntimeError(err.value.decode())
        self.dgks_count += c.value
        return self.dsse(), lin, hin, cut

    def append(self, type, xcol, bcol, h):
        st = ctypes.c_int(0)
        err = ctypes.create_string_buffer(256)
        t = type.encode() if isinstance(type, str) else bytes(type)
        mse = self._L.append(self._h, t, int(xcol), int(bcol), float(h), ctypes.byref(st),
                             err, 256)
        if st.value != 0:
            raise RuntimeError(err.value.decode())
        return mse


def load(kind):
    if kind not in _LIBS:
        _LIBS[kind] = OracleLib(kind)
    return _LIBS[kind]


def marslib_for(kind="port"):
    """A module-like object with the marslib surface over an oracle library."""
    mod = types.SimpleNamespace()
    mod.__version__ = "0.12"

    def _algo(X, y, w, max_terms):
        return OracleAlgo(X, y, w, max_terms, kind=kind)

    mod.MarsAlgo = _algo
    return mod
