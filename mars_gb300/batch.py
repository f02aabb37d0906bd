"""Many independent fits at once (bootstraps, several targets, per-group models).

Each fit is its own handle with its own CUDA stream; ``fit_many`` drives up to
``threads`` fits concurrently from a host thread pool. The C ABI releases the
Python interpreter lock for every call (ctypes), so the fits' kernels overlap
on the device while each fit's host-side decisions (mars.py's epoch loop, the
reference-order append) proceed on its own thread. A single fit of modest n
keeps only a few SMs busy with its dependent FP64 chains; concurrent fits fill
the rest.
"""
import time
from concurrent.futures import ThreadPoolExecutor

from . import marslib
from .mars import forward_pass


def fit_many(problems, threads=16, precision=None, stats=None):
    """Fit every (X, y, w, kwargs) of ``problems`` (w may be None); returns
    (models, seconds per fit) in the input order. ``precision``: 'fp64'
    (default) or 'mixed' for every handle. When ``stats`` is a list, each fit's
    handle counters (marslib.MarsAlgo.stats()) are appended to it, in order."""

    def one(prob):
        X, y, w, kw = prob
        handles = []

        class Lib:
            __version__ = getattr(marslib, "__version__", "0.12")

            @staticmethod
            def MarsAlgo(*a):
                o = marslib.MarsAlgo(*a)
                if precision is not None:
                    o.set_precision(precision)
                handles.append(o)
                return o

        t0 = time.perf_counter()
        model = forward_pass(Lib, X, y, w, **kw)
        dt = time.perf_counter() - t0
        return model, dt, handles[-1].stats() if stats is not None and handles else None

    with ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        out = list(ex.map(one, problems))
    if stats is not None:
        stats.extend(st for _, _, st in out)
    return [m for m, _, _ in out], [t for _, t, _ in out]
