"""Multivariate Adaptive Regression Splines -- GB300 forward pass.

Drop-in for the reference ``mars`` module's forward-pass surface:
``fit`` (mars.py:60-417), ``expand`` (mars.py:423-450) and ``pprint``
(mars.py:741-775). ``fit`` drives ``mars_gb300.marslib.MarsAlgo``, whose
``eval``/``append`` run on the GPU through the C ABI in ``include/mars_gpu.h``.

The epoch loop is the part of the algorithm that decides the selected term
sequence, so it keeps the reference's decision rules exactly: Fast-MARS parent
and input ranking (mars.py:308-316), the mask with the degree/self-interaction
filter (mars.py:237-239, 319-323), first-maximum argmax over (input, parent)
(mars.py:342-343), the GCV choice between a linear term and a hinge pair
(mars.py:349-357), and the stop rules (mars.py:393-406).
"""
import os
import sys
import time

import numpy as np

from . import marslib

__version__ = marslib.__version__
__all__ = ["fit", "expand", "pprint", "__version__"]

MODEL_DTYPE = np.dtype(
    [
        ("type", "S1"),
        ("basis", "i4"),
        ("input", "i4"),
        ("hinge", "f8"),
        ("beta", "f4"),
        ("r2", "f4"),
        ("r2_cv", "f4"),
        ("order", "i4"),
        ("time", "f4"),
    ]
)

def _log_header(logger):
    if logger:
        logger.write("time        #   n    b    x   o    r²    r²_cv\n")
        logger.write("---------- --- --- ---- ---- --  ------ -------\n")


def _log_row(logger, epoch, nbasis, dt, row, labels):
    hh, mm, ss = dt // 3600, (dt // 60) % 60, dt % 60
    logger.write("%02d:%02d:%04.1f " % (hh, mm, ss))
    logger.write("%3d %3d %4d %4d %2d  %6.4f %7.4f" % (
        epoch, nbasis - 1, row["basis"], row["input"], row["order"], row["r2"], row["r2_cv"]))
    if labels is not None:
        width = max(len(s) for s in labels)
        name = ("%%-%ds" % width) % labels[row["input"]]
        if row["type"] == b"l":
            logger.write("  l " + name)
        else:
            logger.write("  h " + name + (" %.4g" % row["hinge"]))
    logger.write("\n")


def _rank_positions(v):
    """Position of each entry in ascending order (0 = smallest)."""
    pos = np.empty_like(v, dtype=np.intp)
    pos[np.argsort(v)] = np.arange(len(v))
    return pos


def fit(X, y, w=None, **kwargs):
    """Forward pass of MARS on the GPU. Same arguments and model array as the
    reference ``mars.fit`` (mars.py:60-175): ``max_terms``, ``max_degree``,
    ``penalty``, ``min_span``, ``tail_span``, ``max_runtime``, ``self_interact``,
    ``linear_only``, ``n_true``, ``logger``, ``callback``, ``r2_window``,
    ``r2_thresh``, ``labels``, ``xfilter``, ``max_basis``, ``max_inputs``,
    ``aging_factor``, ``threads``, ``cuda``. ``threads`` and ``cuda`` are
    accepted for compatibility; candidate evaluation always runs on the GPU.
    """
    return forward_pass(marslib, X, y, w, **kwargs)


def forward_pass(lib, X, y, w=None, **kwargs):
    """The fit loop over any module exposing the ``marslib`` surface."""
    if w is None:
        w = np.ones(len(X), dtype="f")
    X = np.asarray(X)
    y = np.asarray(np.squeeze(y), dtype="f")
    w = np.asarray(np.squeeze(w), dtype="f")

    assert X.dtype == "f", "X data must be 32-bit float"
    assert X.strides[0] == X.itemsize, "X data must be column-major"
    assert y.strides[0] == y.itemsize, "y data must be column-major"
    assert len(X) == len(y) == len(w), "input dataset length mismatch"
    assert len(X) > 0, "empty dataset"

    n, p = X.shape
    opts = dict(
        max_terms=1 + 2 * min(p + n // 20, 15),
        max_degree=3,
        penalty=3.0,
        min_span=None,
        tail_span=0.02,
        max_runtime=48 * 3600,
        self_interact=False,
        linear_only=False,
        n_true=n,
        logger=None,
        callback=None,
        r2_window=32,
        r2_thresh=3e-5,
        labels=None,
        xfilter=lambda x, b: True,
        max_basis=None,
        max_inputs=None,
        aging_factor=1.0,
        threads=-1,
        cuda=False,
    )
    unknown = {k: v for k, v in kwargs.items() if k not in opts}
    if unknown:
        raise TypeError("unknown argument: %s" % unknown)
    opts.update(kwargs)

    t_start = time.time()
    profile = bool(os.environ.get("MARS_CUDA_PROFILE"))
    t_eval = 0.0

    n_true = opts["n_true"]
    penalty = opts["penalty"]
    max_degree = opts["max_degree"]
    self_interact = opts["self_interact"]
    xfilter = opts["xfilter"]
    logger = opts["logger"]
    callback = opts["callback"]
    labels = opts["labels"]

    # Friedman's Eq. (43) default knot spacing (mars.py:225-228).
    min_span = opts["min_span"]
    if min_span is None:
        alpha = 1 / p
        min_span = int(-np.log2(-np.log(1 - alpha) / (n_true * alpha)) / 2.5)
    min_span = max(min_span, 1)

    def dof(m):
        return m + penalty * (m - 1)

    def gcv(mse, m):
        return mse / (1.0 - dof(m) / n_true) ** 2

    def allowed(i, parents):
        return len(parents) < max_degree and (self_interact or i not in parents)

    # The term budget never lets the degrees of freedom reach n_true.
    sizes = np.arange(1, opts["max_terms"] + 1)
    max_terms = sizes[dof(sizes) < n_true].max()

    endspan = max(int(n * opts["tail_span"]), 1)
    algo = lib.MarsAlgo(X, y, w, max_terms)
    var_y = algo.yvar()

    parents_of = [[]]  # input columns used along each basis' parent chain
    epoch = 0
    parent_score = np.array([0.0])
    input_score = np.full(p, np.inf)
    input_seen = np.full(p, epoch)

    model = np.zeros(max_terms, dtype=MODEL_DTYPE)
    model[0] = ("i", 0, 0, np.nan, np.nan, 0, 0, 0, 0)
    _log_header(logger)

    while algo.nbasis() < max_terms:
        # Fast-MARS: rank parents by cached gain, inputs by aged rank.
        use_parents = np.argsort(parent_score)[::-1][: opts["max_basis"]]
        priority = _rank_positions(input_score) + opts["aging_factor"] * (
            epoch - input_seen) * (input_score > 0)
        take = None
        if opts["max_inputs"] is not None:
            take = opts["max_inputs"] + int(np.isinf(input_score).sum())
        use_inputs = np.sort(np.argsort(priority)[::-1][:take])

        mask = np.zeros((p, len(parents_of)), dtype="bool")
        mask[np.ix_(use_inputs, use_parents)] = True
        for i in use_inputs:
            mask[i] &= np.array([allowed(i, b) for b in parents_of])
            mask[i] &= np.array([xfilter(i, b) for b in parents_of])

        t0 = time.perf_counter()
        sse0, sse1, sse2, cut = algo.eval(
            mask, min_span, endspan, opts["linear_only"], opts["threads"], cuda=opts["cuda"])
        t_eval += time.perf_counter() - t0

        active = mask.any(axis=0)
        parent_score[active] = sse2[:, active].max(axis=0)
        input_score[use_inputs] = sse2[use_inputs].max(axis=1)
        input_seen[use_inputs] = epoch
        epoch += 1

        best_lin = np.unravel_index(np.argmax(sse1), sse1.shape)
        best_hinge = np.unravel_index(np.argmax(sse2), sse2.shape)
        dt = time.time() - t_start
        if sse1[best_lin] <= 0 and sse2[best_hinge] <= 0:
            break  # every candidate filtered out or without gain

        m_before = m = algo.nbasis()
        gcv_lin = gcv((1.0 - sse0 - sse1[best_lin]) / n, m + 1)
        gcv_hinge = gcv((1.0 - sse0 - sse2[best_hinge]) / n, m + 2)
        if gcv_lin <= gcv_hinge:
            xcol, bcol, knot = best_lin[0], best_lin[1], np.nan
            kinds = ["l"]
        else:
            xcol, bcol, knot = best_hinge[0], best_hinge[1], cut[best_hinge]
            kinds = ["+", "-"]

        for kind in kinds:
            if algo.nbasis() >= max_terms:
                break  # a hinge pair may only half fit in the budget
            mse = algo.append(kind, xcol, bcol, knot)
            if mse >= 0:
                parents_of.append(parents_of[bcol] + [xcol])
                model[m] = (kind, bcol, xcol, knot, np.nan, 1.0 - mse / var_y,
                            1.0 - gcv(mse, m + 1) / var_y, len(parents_of[-1]), dt)
                parent_score = np.append(parent_score, [0.0])
                m += 1
        assert algo.nbasis() == len(parents_of) == m

        if logger:
            _log_row(logger, epoch, len(parents_of), dt, model[m - 1], labels)
        if callback:
            callback(epoch, len(parents_of), max_terms, model[m - 1])

        if m == m_before:
            break  # no progress: the chosen term was degenerate
        if model[m - 1]["r2"] > 1 - opts["r2_thresh"]:
            break  # essentially perfect fit
        if dt > opts["max_runtime"]:
            break
        window = opts["r2_window"]
        r2cv = model["r2_cv"][: algo.nbasis()]
        if len(r2cv) > window and r2cv[-window:].max() < r2cv.max() - opts["r2_thresh"]:
            break  # no new best GCV R² within the patience window

    if profile:
        total = time.time() - t_start
        share = (100.0 * t_eval / total) if total else 0.0
        sys.stderr.write(
            "[mars] fit: %.2fs total | %.2fs in algo.eval() (%.0f%%) | "
            "%.2fs orchestration (%d epochs)\n" % (total, t_eval, share, total - t_eval, epoch))

    return model[: algo.nbasis()]


def expand(X, model):
    """Basis matrix of ``model`` on ``X`` (mars.py:423-450): column i is its
    parent column times 1 (intercept), x, max(x-h, 0) or max(h-x, 0).
    Returns an (n, len(model)) Fortran-order array of X's dtype."""
    X = np.asarray(X)
    B = np.empty((len(X), len(model)), dtype=X.dtype, order="F")
    for i, node in enumerate(model):
        kind = node["type"]
        kind = kind.decode("utf8") if isinstance(kind, bytes) else kind
        b, x, h = node["basis"], node["input"], node["hinge"]
        if kind == "i":
            B[:, i] = 1.0
            continue
        assert 0 <= x < X.shape[1]
        assert 0 <= b < i
        if kind == "l":
            B[:, i] = B[:, b] * X[:, x]
        elif kind == "+":
            B[:, i] = B[:, b] * np.maximum(X[:, x] - h, 0)
        elif kind == "-":
            B[:, i] = B[:, b] * np.maximum(h - X[:, x], 0)
        else:
            assert False, "unknown basis type %r" % kind
    return B


def pprint(model, beta=None, labels=None):
    """Print one line per basis: coefficient and the product of its factors
    (mars.py:741-775)."""
    if beta is None:
        beta = model["beta"]

    def name(i):
        return labels[i] if labels is not None else "X[%d]" % i

    def factors(i):
        row = model[i]
        if row["type"] == b"+":
            f = "MAX(%s-%g,0)" % (name(row["input"]), row["hinge"])
        elif row["type"] == b"-":
            f = "MAX(%g-%s,0)" % (row["hinge"], name(row["input"]))
        else:
            f = name(row["input"])
        return [f] + factors(row["basis"]) if row["basis"] > 0 else [f]

    for i in range(len(model)):
        line = "  "
        if beta is not None and hasattr(beta, "__getitem__"):
            line += "%+9.4g" % beta[i]
        if model[i]["type"] != b"i":
            line += " * " + " * ".join(factors(i))
        print(line)
