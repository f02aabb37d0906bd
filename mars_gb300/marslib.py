"""``marslib`` surface over the GB300 C ABI (include/mars_gpu.h).

Mirrors the reference pybind11 module (marslib.cc:152-179):
``MarsAlgo(X, y, w, max_terms)`` with ``eval``, ``append``, ``nbasis``,
``yvar`` and ``__version__``, raising ``RuntimeError`` with the reference's
messages. Every call goes to ``lib/libmars_gpu.so``; there is no CPU path,
so a missing library or GPU is an error, never a silent fallback.

Extras over the reference: ``dsse()``, ``set_precision('fp64'|'mixed')``,
``stats()``, ``orth_error()`` (max |Q^T Q - I| and the FP64 RSS) and
``orth_error_by_terms()`` (the same for every leading basis).
"""
import ctypes
import os

import numpy as np

__version__ = "0.12"

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libmars_gpu.so")
PREC_FP64, PREC_MIXED = 0, 1
_lib = None


class Stats(ctypes.Structure):
    _fields_ = [
        ("evals", ctypes.c_longlong),
        ("candidates", ctypes.c_longlong),
        ("knot_evals", ctypes.c_longlong),
        ("dgks_fired", ctypes.c_longlong),
        ("redecided", ctypes.c_longlong),
        ("kernel_launches", ctypes.c_longlong),
        ("h2d_bytes", ctypes.c_longlong),
        ("d2h_bytes", ctypes.c_longlong),
        ("project_flops", ctypes.c_double),
        ("sweep_bytes", ctypes.c_double),
        ("ms_span", ctypes.c_double),
        ("ms_project", ctypes.c_double),
        ("ms_dgks", ctypes.c_double),
        ("ms_normalize", ctypes.c_double),
        ("ms_sweep", ctypes.c_double),
        ("ms_sort", ctypes.c_double),
        ("ms_append", ctypes.c_double),
        ("ms_redecide", ctypes.c_double),
        ("ms_gather", ctypes.c_double),
        ("ms_redecide_gpu", ctypes.c_double),
        ("redecided_flagged", ctypes.c_longlong),
        ("evals_exact", ctypes.c_longlong),
        ("redecided_degenerate", ctypes.c_longlong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def load():
    """Load libmars_gpu.so and bind its C ABI (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(LIB_PATH):
        raise RuntimeError(
            "marslib: %s is not built; run mars_gb300.build.build() (nvcc, sm_103a)" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    vp, sz, i, d = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_double
    fp = ctypes.POINTER(ctypes.c_float)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    lp = ctypes.POINTER(ctypes.c_long)
    bp = ctypes.POINTER(ctypes.c_bool)
    sig = {
        "mars_gpu_last_error": (ctypes.c_char_p, []),
        "mars_gpu_device_count": (i, []),
        "mars_gpu_create": (i, [fp, fp, fp, sz, sz, sz, sz, ctypes.POINTER(vp)]),
        "mars_gpu_destroy": (i, [vp]),
        "mars_gpu_nbasis": (i, [vp, ip]),
        "mars_gpu_yvar": (i, [vp, dp]),
        "mars_gpu_dsse": (i, [vp, dp]),
        "mars_gpu_set_precision": (i, [vp, i]),
        "mars_gpu_eval": (i, [vp, bp, i, i, i, i, i, dp, dp, dp, dp]),
        "mars_gpu_append": (i, [vp, ctypes.c_char, i, i, ctypes.c_float, dp]),
        "mars_gpu_get_stats": (i, [vp, ctypes.POINTER(Stats)]),
        "mars_gpu_orth_error": (i, [vp, dp, dp]),
        "mars_gpu_orth_error_by_terms": (i, [vp, dp, dp, sz, ctypes.POINTER(sz)]),
        "mars_gpu_orthonormalize": (i, [sz, sz, sz, fp, sz, fp, ip, fp, sz, fp, sz, dp, d, lp]),
        "mars_gpu_orthonormalize_col": (i, [sz, sz, dp, fp, sz, d, dp, lp]),
        "mars_gpu_orthonormalize_noalloc": (i, [sz, sz, sz, vp, sz, sz, vp, ip, vp, sz, vp, sz,
                                                vp, d, vp, lp]),
        "mars_gpu_pool_used_bytes": (i, [ctypes.POINTER(sz)]),
        "mars_gpu_gram": (i, [sz, fp, sz, sz, fp, sz, sz, i, dp]),
        "mars_gpu_gram_f64": (i, [sz, dp, sz, sz, dp, sz, sz, i, dp]),
        "mars_gpu_fast_project": (i, [sz, sz, sz, fp, sz, sz, fp, sz, sz, fp, ip, ip, fp, sz, fp,
                                      d, i, i, fp, fp, dp, dp, fp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc):
    if rc != 0:
        raise RuntimeError(load().mars_gpu_last_error().decode())


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _as_f32_vector(a, name):
    if not isinstance(a, np.ndarray) or a.dtype != np.float32:
        raise TypeError("MarsAlgo(): %s must be a float32 numpy array" % name)
    return a


class MarsAlgo:
    """Device-resident forward-pass state (marsalgo.h:16-120)."""

    def __init__(self, X, y, w, max_terms):
        _as_f32_vector(X, "X")
        _as_f32_vector(y, "y")
        _as_f32_vector(w, "w")
        if X.ndim != 2:
            raise RuntimeError("expected 2D array for X")
        if y.ndim != 1:
            raise RuntimeError("expected 1D array for y")
        if w.ndim != 1:
            raise RuntimeError("expected 1D array for w")
        if X.strides[0] != 4:
            raise RuntimeError("X must be column-major")
        if y.strides[0] != 4:
            raise RuntimeError("y must be column-major")
        if w.strides[0] != 4:
            raise RuntimeError("w must be column-major")
        if X.shape[0] != y.shape[0]:
            raise RuntimeError("invalid dimension for y")
        if X.shape[0] != w.shape[0]:
            raise RuntimeError("invalid dimension for w")
        L = load()
        n, p = X.shape
        ldx = X.strides[1] // 4 if p > 1 else n
        h = ctypes.c_void_p()
        check(L.mars_gpu_create(_p(X, ctypes.c_float), _p(y, ctypes.c_float),
                                _p(w, ctypes.c_float), n, p, ldx, int(max_terms), ctypes.byref(h)))
        self._h = h
        self._L = L
        self._p = p
        self._X = X  # borrowed by the library until destroy (keep_alive, marslib.cc:166)
        mode = os.environ.get("MARS_GPU_PRECISION", "").strip().lower()
        if mode:
            self.set_precision(mode)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.mars_gpu_destroy(h)
            self._h = None

    def nbasis(self):
        out = ctypes.c_int()
        check(self._L.mars_gpu_nbasis(self._h, ctypes.byref(out)))
        return out.value

    def yvar(self):
        out = ctypes.c_double()
        check(self._L.mars_gpu_yvar(self._h, ctypes.byref(out)))
        return out.value

    def dsse(self):
        out = ctypes.c_double()
        check(self._L.mars_gpu_dsse(self._h, ctypes.byref(out)))
        return out.value

    def set_precision(self, mode):
        modes = {"fp64": PREC_FP64, "mixed": PREC_MIXED}
        if mode not in modes:
            raise ValueError("precision must be 'fp64' or 'mixed'")
        check(self._L.mars_gpu_set_precision(self._h, modes[mode]))

    def eval(self, mask, min_span, endspan, linear_only, threads, cuda=False):
        """(dsse, linear, hinge, cut) for every (input, parent) pair selected by
        the (p, nbasis) row-major bool `mask` (marslib.cc:41-148). `threads`
        and `cuda` are accepted for compatibility; the GPU evaluates all pairs."""
        if not isinstance(mask, np.ndarray) or mask.dtype != np.bool_:
            raise TypeError("eval(): mask must be a bool numpy array")
        if mask.ndim != 2:
            raise RuntimeError("expected 2D array for mask")
        if mask.strides[1] != 1:
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
        sse0 = ctypes.c_double()
        stride = mask.strides[0] if rows > 0 else m
        check(self._L.mars_gpu_eval(self._h, _p(mask, ctypes.c_bool), rows, stride,
                                    int(min_span), int(endspan), int(bool(linear_only)),
                                    ctypes.byref(sse0), _p(lin, ctypes.c_double),
                                    _p(hin, ctypes.c_double), _p(cut, ctypes.c_double)))
        return sse0.value, lin, hin, cut

    def append(self, type, xcol, bcol, h):
        """Add basis 'l', '+' or '-' (marsalgo.cc:760-875); returns the MSE or -1."""
        t = type.encode() if isinstance(type, str) else bytes(type)
        if len(t) != 1:
            raise RuntimeError("invalid basis type")
        mse = ctypes.c_double()
        check(self._L.mars_gpu_append(self._h, t, int(xcol), int(bcol), float(h),
                                      ctypes.byref(mse)))
        return mse.value

    def stats(self):
        s = Stats()
        check(self._L.mars_gpu_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    def orth_error(self):
        mx, rss = ctypes.c_double(), ctypes.c_double()
        check(self._L.mars_gpu_orth_error(self._h, ctypes.byref(mx), ctypes.byref(rss)))
        return mx.value, rss.value

    def orth_error_by_terms(self):
        """(max |Q_k^T Q_k - I|, 1 - sum(ybo^2)) for every leading basis of
        k + 1 columns, as two float64 arrays of the basis' length."""
        m = self.nbasis()
        mx, rss = np.zeros(m), np.zeros(m)
        count = ctypes.c_size_t()
        dp = ctypes.POINTER(ctypes.c_double)
        check(self._L.mars_gpu_orth_error_by_terms(self._h, mx.ctypes.data_as(dp),
                                                    rss.ctypes.data_as(dp), m,
                                                    ctypes.byref(count)))
        return mx[:count.value], rss[:count.value]


def compiled():
    """The compiled `marslib` extension (mars_gb300/pybind/marslib.cpp), the
    reference's pybind11 module over this library's C ABI. Raises if it was
    not built (no pybind11 headers at build time)."""
    import importlib.machinery
    import importlib.util
    import sysconfig

    path = os.path.join(_HERE, "lib", "marslib" + sysconfig.get_config_var("EXT_SUFFIX"))
    if not os.path.isfile(path):
        raise RuntimeError("the compiled marslib is not built: %s" % path)
    load()  # libmars_gpu.so first, from this directory
    loader = importlib.machinery.ExtensionFileLoader("marslib", path)
    spec = importlib.util.spec_from_loader("marslib", loader)
    mod = importlib.util.module_from_spec(spec)
    loader.exec_module(mod)
    return mod


def device_count():
    return load().mars_gpu_device_count()


def orthonormalize(B, x, mask, Bo, m, tol):
    """Kernel-level mars::orthonormalize on the GPU (kernels.h:52-62).
    B (n, *) column-major f32, Bo (n, >= m) row-major f32. Returns (Bx, s, dgks)."""
    L = load()
    B = np.asfortranarray(B, dtype=np.float32)
    Bo = np.ascontiguousarray(Bo, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    mask = np.ascontiguousarray(mask, dtype=np.int32)
    n, p = B.shape[0], len(mask)
    Bx = np.zeros((n, p), dtype=np.float32, order="F")
    s = np.zeros(p)
    c = ctypes.c_long(0)
    check(L.mars_gpu_orthonormalize(n, m, p, _p(B, ctypes.c_float), n, _p(x, ctypes.c_float),
                                    _p(mask, ctypes.c_int), _p(Bo, ctypes.c_float), Bo.shape[1],
                                    _p(Bx, ctypes.c_float), n, _p(s, ctypes.c_double), tol,
                                    ctypes.byref(c)))
    return Bx, s, c.value


def orthonormalize_col(v, Bo, m, tol):
    """Kernel-level mars::orthonormalize_col on the GPU (kernels.h:91-96).
    Returns (w, v_out, dgks)."""
    L = load()
    v = np.array(v, dtype=np.float64)
    Bo = np.ascontiguousarray(Bo, dtype=np.float32)
    w = ctypes.c_double()
    c = ctypes.c_long(0)
    check(L.mars_gpu_orthonormalize_col(len(v), m, _p(v, ctypes.c_double), _p(Bo, ctypes.c_float),
                                        Bo.shape[1], tol, ctypes.byref(w), ctypes.byref(c)))
    return w.value, v, c.value


def fast_project(B, X, s, cand_x, cand_b, Bo, m, y, tol, use_tc=True, passes=2, timing=None):
    """The fast pass's projection (mars_gpu_fast_project) on host arrays:
    candidate j = B[:, cand_b[j]] * (X[:, cand_x[j]] * s[cand_x[j]]), projected
    off the first m columns of Bo (n, >= m) column-major f32. Returns
    (T (P, m) f32 of the last pass, Bx (n, P) f32 row-major, s, ybx);
    s and ybx are None for passes=1. `timing`, a list, receives the device
    milliseconds of the projection kernels."""
    L = load()
    B = np.asfortranarray(B, dtype=np.float32)
    X = np.asfortranarray(X, dtype=np.float32)
    Bo = np.asfortranarray(Bo, dtype=np.float32)
    s = np.ascontiguousarray(s, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    cx = np.ascontiguousarray(cand_x, dtype=np.int32)
    cb = np.ascontiguousarray(cand_b, dtype=np.int32)
    n, P = B.shape[0], len(cx)
    T = np.empty((P, m), dtype=np.float32)
    Bx = np.empty((n, P), dtype=np.float32)  # row-major, as the fast sweep reads it
    so = np.empty(P)
    yo = np.empty(P)
    ms = ctypes.c_float(0.0)
    check(L.mars_gpu_fast_project(n, m, P, _p(B, ctypes.c_float), n, B.shape[1],
                                  _p(X, ctypes.c_float), n, X.shape[1], _p(s, ctypes.c_float),
                                  _p(cx, ctypes.c_int), _p(cb, ctypes.c_int),
                                  _p(Bo, ctypes.c_float), n, _p(y, ctypes.c_float), float(tol),
                                  int(bool(use_tc)), int(passes), _p(T, ctypes.c_float),
                                  _p(Bx, ctypes.c_float), _p(so, ctypes.c_double),
                                  _p(yo, ctypes.c_double), ctypes.byref(ms)))
    if timing is not None:
        timing.append(ms.value)
    if passes == 1:
        return T, Bx, None, None
    return T, Bx, so, yo


def gram(A, B, exact=False):
    """A.T @ B (A: (n, ka), B: (n, kb), 2-D) with FP64 accumulation over
    128-row chunks on the GPU: float32 inputs (mars_gpu_gram) unless either is
    float64 (mars_gpu_gram_f64); `exact` widens the products and runs the
    chunk chains in FP64."""
    L = load()
    wide = np.asarray(A).dtype == np.float64 or np.asarray(B).dtype == np.float64
    dt, ct = (np.float64, ctypes.c_double) if wide else (np.float32, ctypes.c_float)
    fn = L.mars_gpu_gram_f64 if wide else L.mars_gpu_gram
    A = np.asfortranarray(A, dtype=dt)
    B = np.asfortranarray(B, dtype=dt)
    if A.ndim != 2 or B.ndim != 2 or A.shape[0] != B.shape[0]:
        raise ValueError("shapes are not aligned: %s x %s" % (A.shape, B.shape))
    n, ka = A.shape
    kb = B.shape[1]
    out = np.zeros((ka, kb))
    if ka and kb:
        check(fn(n, _p(A, ct), max(n, 1), ka, _p(B, ct), max(n, 1), kb, int(bool(exact)),
                 _p(out, ctypes.c_double)))
    return out


def pool_used_bytes():
    """Bytes the library's device memory pool has handed out (current device)."""
    L = load()
    v = ctypes.c_size_t(0)
    check(L.mars_gpu_pool_used_bytes(ctypes.byref(v)))
    return v.value


# Limits of the fixed scratch of mars_gpu_orthonormalize_noalloc (mars_gpu.h).
NOALLOC_MAX_CANDIDATES = 4096
NOALLOC_MAX_COEFS = 262144


def orthonormalize_noalloc(n, m, mask, B_ptr, ldB, ncolB, x_ptr, Bo_ptr, ldBo, Bx_ptr, ldBx,
                           s_ptr, tol, stream_ptr=0):
    """mars_gpu_orthonormalize on caller-owned device arrays (integer device
    addresses), queued on `stream_ptr` (a cudaStream_t; 0 = default stream),
    with no device allocation. mask is a host int array of parent columns,
    each below ncolB (the columns of B). Returns the number of columns DGKS
    retried."""
    L = load()
    mask = np.ascontiguousarray(mask, dtype=np.int32)
    c = ctypes.c_long(0)
    check(L.mars_gpu_orthonormalize_noalloc(n, m, len(mask), B_ptr, ldB, ncolB, x_ptr,
                                            _p(mask, ctypes.c_int), Bo_ptr, ldBo, Bx_ptr, ldBx,
                                            s_ptr or None, tol, stream_ptr or None,
                                            ctypes.byref(c)))
    return c.value
