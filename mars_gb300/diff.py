"""Differentiable prediction of a fitted model, for post-search knot refinement.

``predict(X, model, beta, knots)`` is a ``torch.autograd.Function`` over the
CUDA kernels ``mars_gpu_expand`` / ``mars_gpu_expand_backward``
(include/mars_gpu.h): the basis of ``mars.expand`` (mars.py:423-450) times
``beta``, with gradients with respect to ``X``, ``beta`` and the continuous
hinge knots. ``refine_knots`` moves the knots of a fitted model by Adam on the
residual sum of squares. Torch provides the device memory and the stream; the
arithmetic is in the kernels.
"""
import ctypes

import numpy as np

from . import marslib

KIND = {b"i": 0, b"l": 1, b"+": 2, b"-": 3, "i": 0, "l": 1, "+": 2, "-": 3}


def _lib():
    L = marslib.load()
    if not getattr(L, "_expand_bound", False):
        vp, sz, i = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
        L.mars_gpu_expand_workspace.restype = sz
        L.mars_gpu_expand_workspace.argtypes = [sz, i]
        L.mars_gpu_expand.restype = i
        L.mars_gpu_expand.argtypes = [vp, vp, vp, vp, vp, i, vp, sz, sz, vp, vp, sz, vp]
        L.mars_gpu_expand_backward.restype = i
        L.mars_gpu_expand_backward.argtypes = [vp, vp, vp, vp, vp, i, vp, sz, sz, vp, vp, sz,
                                               vp, vp, vp, vp]
        L._expand_bound = True
    return L


def terms_of(model):
    """(kind, parent, input) int32 arrays and the knots (NaN -> 0) of a model."""
    kind = np.array([KIND[t] for t in model["type"]], dtype=np.int32)
    parent = np.ascontiguousarray(model["basis"], dtype=np.int32)
    inp = np.ascontiguousarray(model["input"], dtype=np.int32)
    knots = np.ascontiguousarray(np.nan_to_num(np.asarray(model["hinge"], dtype=np.float64)),
                                 dtype=np.float32)
    return kind, parent, inp, knots


def _colmajor(X):
    """X as an (N, p) column-major float32 CUDA tensor (a view when it is one)."""
    if X.dim() != 2:
        raise ValueError("X must be 2-D")
    if X.stride(0) == 1 and X.stride(1) >= X.shape[0]:
        return X
    return X.t().contiguous().t()


def _stream_ptr(torch, device):
    return torch.cuda.current_stream(device).cuda_stream


class _Expand:
    """Holder of the torch.autograd.Function (torch is imported lazily)."""

    fn = None


def _function():
    if _Expand.fn is not None:
        return _Expand.fn
    import torch

    class ExpandPredict(torch.autograd.Function):
        @staticmethod
        def forward(ctx, X, beta, knots, kind, parent, inp):
            Xc = _colmajor(X.detach())
            N = Xc.shape[0]
            M = kind.numel()
            pred = torch.empty(N, dtype=torch.float32, device=X.device)
            L = _lib()
            rc = L.mars_gpu_expand(kind.data_ptr(), parent.data_ptr(), inp.data_ptr(),
                                   knots.data_ptr(), beta.data_ptr(), M, Xc.data_ptr(),
                                   Xc.stride(1), N, pred.data_ptr(), None, N,
                                   _stream_ptr(torch, X.device))
            marslib.check(rc)
            ctx.save_for_backward(Xc, beta, knots, kind, parent, inp)
            return pred

        @staticmethod
        def backward(ctx, g):
            Xc, beta, knots, kind, parent, inp = ctx.saved_tensors
            N, M = Xc.shape[0], kind.numel()
            g = g.contiguous().to(torch.float32)
            L = _lib()
            ws = torch.empty(max(1, L.mars_gpu_expand_workspace(N, M)), dtype=torch.uint8,
                             device=Xc.device)
            dbeta = torch.empty(M, dtype=torch.float64, device=Xc.device)
            dknot = torch.empty(M, dtype=torch.float64, device=Xc.device)
            dX = None
            if ctx.needs_input_grad[0]:
                dXt = torch.zeros((Xc.shape[1], N), dtype=torch.float32, device=Xc.device)
                dX = dXt.t()
            rc = L.mars_gpu_expand_backward(kind.data_ptr(), parent.data_ptr(), inp.data_ptr(),
                                            knots.data_ptr(), beta.data_ptr(), M, Xc.data_ptr(),
                                            Xc.stride(1), N, g.data_ptr(),
                                            None if dX is None else dX.data_ptr(), N,
                                            dbeta.data_ptr(), dknot.data_ptr(), ws.data_ptr(),
                                            _stream_ptr(torch, Xc.device))
            marslib.check(rc)
            return (dX, dbeta.to(beta.dtype), dknot.to(knots.dtype), None, None, None)

    _Expand.fn = ExpandPredict
    return ExpandPredict


def predict(X, model, beta=None, knots=None):
    """pred = expand(X, model) @ beta on the GPU, differentiable in X, beta
    and knots (CUDA float32 tensors; beta/knots default to the model's)."""
    import torch

    kind, parent, inp, k0 = terms_of(model)
    dev = X.device
    if beta is None:
        beta = torch.as_tensor(np.ascontiguousarray(np.nan_to_num(model["beta"]), np.float32),
                               device=dev)
    if knots is None:
        knots = torch.as_tensor(k0, device=dev)
    t = lambda a: torch.as_tensor(a, device=dev)  # noqa: E731
    return _function().apply(X, beta, knots, t(kind), t(parent), t(inp))


def fit_beta(X, y, model, knots=None):
    """Least-squares coefficients of the model's basis (f64 solve of the f32 basis)."""
    import torch

    kind, parent, inp, k0 = terms_of(model)
    dev = X.device
    if knots is None:
        knots = torch.as_tensor(k0, device=dev)
    Xc = _colmajor(X.detach())
    N, M = Xc.shape[0], kind.numel() if hasattr(kind, "numel") else len(kind)
    Bt = torch.empty((M, N), dtype=torch.float32, device=dev)
    L = _lib()
    t = lambda a: torch.as_tensor(a, device=dev)  # noqa: E731
    tk, tp, ti = t(kind), t(parent), t(inp)
    ones = torch.ones(M, dtype=torch.float32, device=dev)
    rc = L.mars_gpu_expand(tk.data_ptr(), tp.data_ptr(), ti.data_ptr(), knots.data_ptr(),
                           ones.data_ptr(), M, Xc.data_ptr(), Xc.stride(1), N, None,
                           Bt.data_ptr(), N, _stream_ptr(torch, dev))
    marslib.check(rc)
    B = Bt.t().to(torch.float64)
    sol = torch.linalg.lstsq(B, y.to(torch.float64).reshape(-1, 1)).solution
    return sol.reshape(-1).to(torch.float32)


def refine_knots(X, y, model, steps=200, lr=1e-3, beta=None):
    """Adam on sum((pred - y)^2) over beta and the hinge knots. Returns
    (knots, beta, rss history) as tensors / a list."""
    import torch

    kind, _, _, k0 = terms_of(model)
    dev = X.device
    knots = torch.nn.Parameter(torch.as_tensor(k0, device=dev).clone())
    if beta is None:
        beta = fit_beta(X, y, model)
    beta = torch.nn.Parameter(beta.detach().clone())
    opt = torch.optim.Adam([beta, knots], lr=lr)
    hinge = torch.as_tensor(np.isin(kind, (2, 3)), device=dev)
    hist = []
    for _ in range(steps):
        opt.zero_grad()
        r = predict(X, model, beta, knots) - y
        loss = (r.double() * r.double()).sum()
        loss.backward()
        knots.grad.mul_(hinge)  # only hinge terms have a knot
        opt.step()
        hist.append(float(loss.detach()))
    return knots.detach(), beta.detach(), hist
