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
import io
import os
import sys
import time

import numpy as np

from . import marslib

__version__ = marslib.__version__
__all__ = ["fit", "expand", "pprint", "gram", "prune", "compact", "dumps", "loads", "save",
           "load", "__version__"]

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


# ---------------------------------------------------------------------------
# Backward pass (mars.py:456-695): Gram matrices on the GPU, then backward
# elimination by rank-1 Schur downdates of the inverse Gram matrix.
# ---------------------------------------------------------------------------
def gram(A, B=None):
    """A.T @ B (A.T @ A when B is None) with float64 accumulation over
    128-row chunks, on the GPU in the reference's arithmetic (mars.py:456-490;
    mars_gpu_gram, or mars_gpu_gram_f64 for float64 inputs). 1-D
    arguments are columns; the result is a float when both are 1-D, 1-D when
    one is, else 2-D."""
    if B is None:
        B = A
    A = np.asarray(A)
    B = np.asarray(B)
    if len(A) != len(B):
        raise ValueError("shapes are not aligned: %s x %s" % (A.shape, B.shape))
    A2 = A.reshape(len(A), -1) if A.ndim == 1 else A
    B2 = B.reshape(len(B), -1) if B.ndim == 1 else B
    # matrix-matrix products in the reference's chunk arithmetic; products with
    # a vector (its BLAS uses another order there) exactly, in FP64
    out = marslib.gram(A2, B2, exact=A.ndim == 1 or B.ndim == 1)
    if A.ndim == 1 and B.ndim == 1:
        return float(out[0, 0])
    if A.ndim == 1:
        return out[0]
    if B.ndim == 1:
        return out[:, 0]
    return out


def _cholesky_inverse(XX, XY, YY, idx, ridge):
    """(H, beta, SSE) on the active columns idx: H the inverse of the loaded
    Gram block, beta = H XY, SSE = YY - XY . beta (mars.py:496-544). A block
    that is not numerically positive definite gets a last-resort diagonal
    jitter, so H stays a true inverse."""
    import scipy.linalg

    m = len(idx)
    if m == 0:
        return np.zeros((0, 0)), np.zeros(0), float(YY)
    G = XX[np.ix_(idx, idx)]
    g = XY[idx]
    if ridge > 0:
        G = G + ridge * np.eye(m)
    try:
        L = np.linalg.cholesky(G)
    except np.linalg.LinAlgError:
        L = np.linalg.cholesky(G + 1e-8 * (np.trace(G) / m + 1.0) * np.eye(m))
    factor = (L, True)
    beta = scipy.linalg.cho_solve(factor, g)
    H = scipy.linalg.cho_solve(factor, np.eye(m))
    return H, beta, max(float(YY - g @ beta), 0.0)


def _eliminate(XX, XY, YY, mask, penalty, n_true, ridge=0.0):
    """Backward stepwise selection (mars.py:547-619): repeatedly drop the
    active column with the least SSE increase beta_j^2 / H_jj (never the
    intercept, global column 0), downdating H and beta by a rank-1 Schur
    complement, refreshing them from a Cholesky every max(64, M/4) drops,
    and keep the subset with the best GCV seen."""
    M = len(XX)
    idx = np.flatnonzero(mask)
    if len(idx) == 0:
        return mask.copy()
    H, beta, sse = _cholesky_inverse(XX, XY, YY, idx, ridge)

    def gcv(v, m):
        d = 1.0 - (m + penalty * (m - 1)) / n_true
        return v / (d * d) if d > 0 else np.inf

    best, keep = gcv(sse, len(idx)), mask.copy()
    cur = mask.copy()
    refresh, since = max(64, M // 4), 0
    while len(idx):
        h = np.diag(H)
        floor = 1e-12 * max(float(h.max()), 1.0)
        cost = np.full(len(beta), np.inf)
        np.divide(beta * beta, h, out=cost, where=h > floor)
        if idx[0] == 0:
            cost[0] = np.inf  # the intercept stays
        j = int(np.argmin(cost))
        if not np.isfinite(cost[j]):
            break
        sse += max(float(cost[j]), 0.0)
        col = H[:, j]
        v = col / H[j, j]
        beta = beta - beta[j] * v
        H = H - np.outer(v, col)
        H = 0.5 * (H + H.T)
        np.fill_diagonal(H, np.maximum(np.diag(H), 0.0))
        beta = np.delete(beta, j)
        H = np.delete(np.delete(H, j, axis=0), j, axis=1)
        cur[idx[j]] = False
        idx = np.delete(idx, j)
        since += 1
        if since >= refresh and len(idx):
            H, beta, sse = _cholesky_inverse(XX, XY, YY, idx, ridge)
            since = 0
        g = gcv(sse, len(idx))
        if g < best:
            best, keep = g, cur.copy()
    return keep


def prune(B, y, w=None, n_true=None, penalty=3.0, ridge=0.0, mask=None):
    """Coefficients of the basis B (n, M) by backward stepwise selection with
    GCV (mars.py:622-695; Friedman 1991, section 3.4): the intercept column 0
    is never dropped, columns are standardised to a unit Gram diagonal (so
    `ridge` acts alike on every column), pruned terms get coefficient 0, and
    the result is in the original scale. The Gram matrices run on the GPU."""
    B = np.asarray(B)
    y = np.asarray(y)
    n, M = B.shape
    if n_true is None:
        n_true = n
    bad = ~np.isfinite(y)
    if bad.any():
        w = np.ones(len(y), dtype=B.dtype) if w is None else np.asarray(w)
        w = np.where(bad, 0, w)
        y = np.where(bad, 0, y)
    if w is not None:
        root = np.sqrt(np.asarray(w, dtype=B.dtype))
        B = B * root[:, None]
        y = y * root
    XX = gram(B)
    XY = gram(B, y)
    YY = gram(y, y)
    d = np.sqrt(np.diag(XX))
    live = d > 0
    scale = np.where(live, d, 1.0)
    XX = XX / scale / scale[:, None]
    XY = XY / scale
    mask = (np.array(mask) if mask is not None else np.ones(M, dtype=bool)) & live
    chosen = _eliminate(XX, XY, YY, mask, penalty, n_true, ridge)
    if ridge > 0:
        XX = XX + ridge * np.eye(M)
    beta = np.zeros(M)
    if chosen.any():
        beta[chosen] = np.linalg.lstsq(XX[np.ix_(chosen, chosen)], XY[chosen], rcond=None)[0]
    return beta / scale


# ---------------------------------------------------------------------------
# Model surgery and storage (mars.py:701-735; the model dtype, mars.py:261-274)
# ---------------------------------------------------------------------------
def compact(model):
    """The model without its pruned terms (beta == 0), keeping every ancestor
    a kept term needs (with its beta, possibly 0) and renumbering the parent
    pointers (mars.py:701-735)."""
    keep = np.asarray(model["beta"]) != 0
    for i in range(len(model) - 1, 0, -1):  # parents precede their children
        if keep[i] and model[i]["type"] != b"i":
            keep[model[i]["basis"]] = True
    where = np.full(len(model), -1, dtype="i4")
    where[keep] = np.arange(int(keep.sum()), dtype="i4")
    out = model[keep].copy()
    out["basis"] = where[out["basis"]]
    return out


def _checked(model):
    model = np.asarray(model)
    if model.dtype != MODEL_DTYPE or model.ndim != 1:
        raise ValueError("not a MARS model array (dtype %s)" % (model.dtype,))
    return model


def dumps(model):
    """The model as bytes: the .npy encoding of its structured array (the
    model dtype, little-endian), no pickling."""
    buf = io.BytesIO()
    np.save(buf, np.ascontiguousarray(_checked(model)), allow_pickle=False)
    return buf.getvalue()


def loads(data):
    """A model from dumps() bytes; the dtype is checked."""
    return _checked(np.load(io.BytesIO(data), allow_pickle=False))


def save(path, model):
    with open(path, "wb") as f:
        f.write(dumps(model))


def load(path):
    with open(path, "rb") as f:
        return loads(f.read())


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
