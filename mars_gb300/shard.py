"""One fit over several GPUs: the candidates of every epoch sharded by input
column, the basis replicated.

Within an epoch the (input, parent) candidates are independent
(marsalgo.cc:402-662 evaluates them per input column; marslib.cc:100-136 runs
those columns as an OpenMP loop). Rank r of a world of W owns the contiguous
block of input columns [r p / W, (r + 1) p / W) and evaluates only those rows
of the mask; its handle still holds the whole basis, because every rank
appends the same term with the same reference-order arithmetic, so the bases
stay identical bit for bit without being sent.

The per-epoch exchange is one all-gather of each rank's (linear, hinge, cut)
rows -- p x m float64 values in all -- after which every rank holds the full
arrays the single-GPU eval returns, entry for entry (each is computed by its
owner alone and copied, not summed). The fit loop then takes the first
maximum in row-major order (mars.py:342-343), which is the deterministic
tie-break by lowest (input, parent), and every rank reaches the same decision.

``sharded(lib, group)`` wraps any module with the marslib surface (the GPU
binding, or in tests the CPU oracle) into one whose MarsAlgo does this over a
torch.distributed process group (gloo for host tensors; an NCCL group gets
device tensors).
"""
import types

import numpy as np


def owned_columns(p, rank, world):
    """[lo, hi): the input columns rank `rank` of `world` evaluates."""
    return (p * rank) // world, (p * (rank + 1)) // world


def combine(parts, p):
    """The full (p, m) arrays from every rank's (lo, hi, linear, hinge, cut)
    rows, each entry taken from the rank that owns its input column."""
    m = parts[0][2].shape[1]
    lin = np.zeros((p, m))
    hin = np.zeros((p, m))
    cut = np.full((p, m), np.nan)
    for lo, hi, li, hi_, cu in parts:
        lin[lo:hi] = li
        hin[lo:hi] = hi_
        cut[lo:hi] = cu
    return lin, hin, cut


class _Exchange:
    """All-gather of fixed-shape float64 blocks over a process group."""

    def __init__(self, group=None):
        import torch
        import torch.distributed as dist

        self.torch, self.dist, self.group = torch, dist, group
        self.world = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        backend = dist.get_backend(group)
        self.device = torch.device("cuda", torch.cuda.current_device()) \
            if backend == "nccl" else torch.device("cpu")

    def gather(self, block):
        t = self.torch.from_numpy(np.ascontiguousarray(block)).to(self.device)
        out = [self.torch.empty_like(t) for _ in range(self.world)]
        self.dist.all_gather(out, t, group=self.group)
        return [o.cpu().numpy() for o in out]


def sharded(lib, group=None):
    """A marslib-like module whose MarsAlgo evaluates this rank's input
    columns on `lib.MarsAlgo` and exchanges the results (module docstring)."""
    ex = _Exchange(group)

    class ShardedAlgo:
        def __init__(self, X, y, w, max_terms):
            self._inner = lib.MarsAlgo(X, y, w, max_terms)
            self._p = X.shape[1]
            self.lo, self.hi = owned_columns(self._p, ex.rank, ex.world)

        def __getattr__(self, k):
            return getattr(self._inner, k)

        def eval(self, mask, min_span, endspan, linear_only, threads, cuda=False):
            mask = np.asarray(mask)
            rows = mask.shape[0]
            mine = np.zeros_like(mask)
            lo, hi = min(self.lo, rows), min(self.hi, rows)
            mine[lo:hi] = mask[lo:hi]
            sse0, lin, hin, cut = self._inner.eval(mine, min_span, endspan, linear_only,
                                                   threads, cuda)
            m = lin.shape[1]
            # fixed-shape block: this rank's rows, padded to the largest share
            share = -(-self._p // ex.world)
            block = np.zeros((3, share, m))
            block[0, :hi - lo] = lin[lo:hi]
            block[1, :hi - lo] = hin[lo:hi]
            block[2, :hi - lo] = cut[lo:hi]
            parts = []
            for r, b in enumerate(ex.gather(block)):
                rlo, rhi = owned_columns(self._p, r, ex.world)
                rlo, rhi = min(rlo, rows), min(rhi, rows)
                k = rhi - rlo
                parts.append((rlo, rhi, b[0, :k], b[1, :k], b[2, :k]))
            full = combine(parts, rows)
            return (sse0,) + full

    mod = types.SimpleNamespace(MarsAlgo=ShardedAlgo, __version__=getattr(lib, "__version__", ""))
    return mod
