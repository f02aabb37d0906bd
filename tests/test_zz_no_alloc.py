"""mars_gpu_orthonormalize_noalloc: the candidate projection on caller-owned
device arrays with its scratch in fixed module-scope device memory.

Compared with the allocating entry point mars_gpu_orthonormalize on the same
inputs, twice in a row on the same buffers (the scratch is reused, nothing in
it may be assumed zero). Both run the same kernels in the same order, so the
tolerance is zero: the outputs must be bitwise equal.
"""
import numpy as np
import pytest

from tests.scenarios import make_orthonormal_basis

pytestmark = pytest.mark.gpu


def _problem(seed):
    """A DGKS-triggering column, an exactly degenerate one and mixed
    magnitudes (the shape of the reference's test_kernels.cc:369-525)."""
    rng = np.random.default_rng(seed)
    n, m, p, tol = 8192, 96, 40, 1e-14
    Bo = make_orthonormal_basis(n, m, rng)
    Q = Bo.astype(np.float64)
    B = rng.uniform(-1, 1, (n, m)).astype(np.float32)
    B *= (2.0 ** (np.arange(m) % 5)).astype(np.float32)
    v = rng.uniform(-1, 1, n)
    v -= Q @ (Q.T @ v)
    v /= np.linalg.norm(v)
    B[:, 3] = (np.sqrt(0.97) * Q[:, 0] + np.sqrt(0.03) * v).astype(np.float32)
    B[:, 7] = Bo[:, 1]
    mask = np.sort(rng.choice(m, p, replace=False)).astype(np.int32)
    mask[:2] = [3, 7]
    mask.sort()
    x = rng.uniform(0.5, 1.5, n).astype(np.float32)
    return np.asfortranarray(B), x, mask, Bo, m, tol


def _noalloc(torch, lib, B, x, mask, Bo, m, tol, stream):
    dev = torch.device("cuda", 0)
    n, p = B.shape[0], len(mask)
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).to(dev)  # column-major (n, *) as rows
    dx = torch.from_numpy(x).to(dev)
    dBo = torch.from_numpy(Bo).to(dev)
    dBx = torch.full((p, n), float("nan"), dtype=torch.float32, device=dev)
    ds = torch.full((p,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    outs = []
    for _ in range(2):
        dgks = lib.orthonormalize_noalloc(n, m, mask, dB.data_ptr(), n, B.shape[1], dx.data_ptr(),
                                          dBo.data_ptr(), Bo.shape[1], dBx.data_ptr(), n,
                                          ds.data_ptr(), tol, stream.cuda_stream)
        stream.synchronize()
        outs.append((dBx.cpu().numpy().T.copy(), ds.cpu().numpy().copy(), dgks))
    return outs


@pytest.mark.parametrize("seed", [0, 1])
def test_noalloc_matches_allocating_entry_point(gpu, seed):
    import torch

    from mars_gb300 import marslib

    B, x, mask, Bo, m, tol = _problem(seed)
    Bx_ref, s_ref, dgks_ref = marslib.orthonormalize(B, x, mask, Bo, m, tol)
    assert dgks_ref >= 1
    stream = torch.cuda.Stream(device=0)
    for Bx, s, dgks in _noalloc(torch, marslib, B, x, mask, Bo, m, tol, stream):
        np.testing.assert_array_equal(Bx, Bx_ref)
        np.testing.assert_array_equal(s, s_ref)
        assert dgks == dgks_ref


def test_noalloc_default_stream_and_null_s(gpu):
    import torch

    from mars_gb300 import marslib

    B, x, mask, Bo, m, tol = _problem(2)
    Bx_ref, _, _ = marslib.orthonormalize(B, x, mask, Bo, m, tol)
    dev = torch.device("cuda", 0)
    n, p = B.shape[0], len(mask)
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).to(dev)
    dx = torch.from_numpy(x).to(dev)
    dBo = torch.from_numpy(Bo).to(dev)
    dBx = torch.zeros((p, n), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    marslib.orthonormalize_noalloc(n, m, mask, dB.data_ptr(), n, B.shape[1], dx.data_ptr(),
                                   dBo.data_ptr(), Bo.shape[1], dBx.data_ptr(), n, 0, tol, 0)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(0)[0]
    pool_before = marslib.pool_used_bytes()
    marslib.orthonormalize_noalloc(n, m, mask, dB.data_ptr(), n, B.shape[1], dx.data_ptr(),
                                   dBo.data_ptr(), Bo.shape[1], dBx.data_ptr(), n, 0, tol, 0)
    torch.cuda.synchronize()
    # no device allocation in the call: neither from the driver nor from the
    # library's own pool (which keeps freed memory cached, so a pool
    # allocation would not show in the free device memory)
    assert torch.cuda.mem_get_info(0)[0] == free_before
    assert marslib.pool_used_bytes() == pool_before
    np.testing.assert_array_equal(dBx.cpu().numpy().T, Bx_ref)


def test_noalloc_rejects_oversize(gpu):
    import torch

    from mars_gb300 import marslib

    dev = torch.device("cuda", 0)
    n = 64
    buf = torch.zeros(n * 8, dtype=torch.float32, device=dev)
    ptr = buf.data_ptr()
    too_many = np.zeros(marslib.NOALLOC_MAX_CANDIDATES + 1, np.int32)
    with pytest.raises(RuntimeError, match="too many candidate columns"):
        marslib.orthonormalize_noalloc(n, 1, too_many, ptr, n, 1, ptr, ptr, 1, ptr, n, 0, 1e-14)
    m = marslib.NOALLOC_MAX_COEFS // 64 + 1
    with pytest.raises(RuntimeError, match="exceeds the fixed scratch"):
        marslib.orthonormalize_noalloc(n, m, np.zeros(64, np.int32), ptr, n, 1, ptr, ptr, m, ptr,
                                       n, 0, 1e-14)
    # a parent index past the columns of B is refused before any device access
    with pytest.raises(RuntimeError, match="outside the columns of B"):
        marslib.orthonormalize_noalloc(n, 1, np.array([0, 8], np.int32), ptr, n, 8, ptr, ptr, 1,
                                       ptr, n, 0, 1e-14)
