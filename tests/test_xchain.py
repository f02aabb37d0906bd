"""The chunked exact accumulation (mars_gb300/csrc/xchain.cuh) on the host.

The kernels that replace the reference's sequential FP64 column chains
(kernels.cc:215-237, kernels.cc:361-366, marsalgo.cc:359-369) cut the rows into
chunks, run each chunk speculatively from a guessed entry value, and walk the
chunks once. tests/xchain_host.cpp builds the same header on the host; these
tests check its result against the recurrence as written, bit for bit, on data
chosen to break each of the checks: ties, binade crossings, sign changes, exact
zeros, subnormals, NaN and infinities, and guesses that are wrong on purpose.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def xlib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("xchain") / "xchain_host.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
                    "-o", out, os.path.join(HERE, "xchain_host.cpp")], check=True)
    lib = ctypes.CDLL(out)
    fp = ctypes.POINTER(ctypes.c_float)
    lib.xc_host_sequential.restype = ctypes.c_double
    lib.xc_host_sequential.argtypes = [fp, fp, ctypes.c_int]
    lib.xc_host_chunked.restype = ctypes.c_double
    lib.xc_host_chunked.argtypes = [fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    lib.xc_host_sequential_d.restype = ctypes.c_double
    lib.xc_host_sequential_d.argtypes = [fp, dp, ctypes.c_int]
    lib.xc_host_composed.restype = ctypes.c_double
    lib.xc_host_composed.argtypes = [fp, dp, ctypes.c_int, ctypes.c_int, ip, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_double, ip, ip, ip]
    for name in ("xc_host_kernel4", "xc_host_kernel8"):
        getattr(lib, name).restype = ctypes.c_double
        getattr(lib, name).argtypes = [fp, dp, ctypes.c_int, ctypes.c_int, ip, ip]
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def run(lib, a, b, K, mode=0, scale=0.0):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    n = a.size
    re = ctypes.c_int(0)
    want = lib.xc_host_sequential(_ptr(a), _ptr(b), n)
    got = lib.xc_host_chunked(_ptr(a), _ptr(b), n, K, mode, scale, ctypes.byref(re))
    return want, got, re.value


def same(x, y):
    return np.array(x, np.float64).view(np.uint64) == np.array(y, np.float64).view(np.uint64)


def cases(seed=0):
    r = np.random.default_rng(seed)
    n = 20000
    z = r.standard_normal(n).astype(np.float32)
    yield "signed", z, r.standard_normal(n).astype(np.float32)
    yield "squares", z, z
    yield "positive", np.abs(z), np.abs(r.standard_normal(n)).astype(np.float32)
    # a head of 1.5 * 2^54 (ulp 4) then small integers: every step rounds and a
    # quarter of them are exact ties
    big = r.integers(1, 1 << 12, n).astype(np.float32)
    big[0] = 1.5 * 2.0 ** 24
    one = np.ones(n, np.float32)
    one[0] = 2.0 ** 30
    yield "ties", big, one
    # quantised data: products are short dyadics
    q = (r.integers(-64, 64, n) / 16).astype(np.float32)
    yield "quantised", q, (r.integers(-8, 8, n) / 4).astype(np.float32)
    # exponents spread over +-40 binades
    w = (r.standard_normal(n) * 2.0 ** r.integers(-40, 40, n)).astype(np.float32)
    yield "wide", w, r.standard_normal(n).astype(np.float32)
    # exact cancellation back to zero
    c = np.repeat(r.standard_normal(n // 2).astype(np.float32), 2)
    s = np.tile(np.array([1, -1], np.float32), n // 2)
    yield "cancel", c, s
    # drifting across many binades, both signs
    d = (np.linspace(-3, 3, n) ** 3).astype(np.float32)
    yield "drift", d, np.ones(n, np.float32)
    # subnormal products
    t = (r.standard_normal(n) * 1e-20).astype(np.float32)
    yield "tiny", t, (r.standard_normal(n) * 1e-20).astype(np.float32)


@pytest.mark.parametrize("K", [1, 2, 7, 32, 160, 1024])
def test_chunked_equals_sequential(xlib, K):
    for name, a, b in cases():
        want, got, _ = run(xlib, a, b, K)
        assert same(want, got), (name, K, want, got)


@pytest.mark.parametrize("mode,scale", [(1, 1e-9), (1, 1e-3), (1, -0.5), (2, 1.0),
                                        (2, -3.0), (2, 2.0), (2, 1e6), (3, 0.0),
                                        (3, 1.0), (3, -7.5), (3, float("inf")),
                                        (3, float("nan"))])
def test_wrong_guesses_are_caught(xlib, mode, scale):
    for name, a, b in cases(1):
        want, got, _ = run(xlib, a, b, 64, mode, scale)
        assert same(want, got), (name, mode, scale, want, got)


def test_special_values(xlib):
    r = np.random.default_rng(2)
    n = 5000
    for bad in (np.nan, np.inf, -np.inf):
        a = r.standard_normal(n).astype(np.float32)
        a[n // 3] = bad
        want, got, _ = run(xlib, a, np.ones(n, np.float32), 50)
        assert same(want, got) or (np.isnan(want) and np.isnan(got)), (bad, want, got)
    for n in (0, 1, 2, 3, 31, 33):
        a = r.standard_normal(n).astype(np.float32)
        for K in (1, 2, 5, 64):
            want, got, _ = run(xlib, a, a, K)
            assert same(want, got), (n, K)


def test_few_chunks_are_redone(xlib):
    """With the kernel's guesses a sum of squares re-runs (almost) no chunk; a signed
    random walk re-runs the chunks where it climbs two binades from near zero (a
    change of sign alone is translated)."""
    r = np.random.default_rng(3)
    n = 200000
    z = r.standard_normal(n).astype(np.float32)
    want, got, redone = run(xlib, z, z, 1024)
    assert same(want, got)
    assert redone <= 4, redone
    want, got, redone = run(xlib, z, r.standard_normal(n).astype(np.float32), 1024)
    assert same(want, got)
    assert redone <= 60, redone


def composed(lib, a, b, K, fan, mode=0, scale=0.0):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float64)
    f = (ctypes.c_int * max(1, len(fan)))(*fan)
    re, de = ctypes.c_int(0), ctypes.c_int(0)
    built = (ctypes.c_int * 2)()
    fp = ctypes.POINTER(ctypes.c_float)
    dp = ctypes.POINTER(ctypes.c_double)
    want = lib.xc_host_sequential_d(a.ctypes.data_as(fp), b.ctypes.data_as(dp), a.size)
    got = lib.xc_host_composed(a.ctypes.data_as(fp), b.ctypes.data_as(dp), a.size, K, f,
                               len(fan), mode, scale, ctypes.byref(re), ctypes.byref(de), built)
    return want, got, re.value, de.value


# the append kernel's levels: 8 chunks, 4 sub-groups, 8 warps, groups of 16 blocks
FANS = [[], [2], [8, 4], [8, 4, 8, 16], [3, 5, 2]]


@pytest.mark.parametrize("K", [1, 7, 64, 256, 1000, 4096])
def test_composed_equals_sequential(xlib, K):
    """Records composed level by level and walked with descents give the
    sequential chain bit for bit, with f32 x f64 terms (the Gram-Schmidt
    chains of the append)."""
    r = np.random.default_rng(K)
    for fan in FANS:
        for name, a, b in cases(K):
            bd = b.astype(np.float64)
            if name in ("signed", "wide"):
                bd = bd * (1.0 + 2.0 ** -30 * r.standard_normal(bd.size))  # full f64 mantissas
            want, got, _, _ = composed(xlib, a, bd, K, fan)
            assert same(want, got) or (np.isnan(want) and np.isnan(got)), (name, K, fan)


@pytest.mark.parametrize("mode,scale", [(1, 1e-9), (1, -0.5), (2, 3.0), (2, -1e6), (3, 0.0),
                                        (3, 2.5), (3, float("nan"))])
def test_composed_wrong_guesses(xlib, mode, scale):
    for name, a, b in cases(2):
        want, got, _, _ = composed(xlib, a, b.astype(np.float64), 512, [8, 4, 8], mode, scale)
        assert same(want, got) or (np.isnan(want) and np.isnan(got)), (name, mode, scale)


def test_composed_special_values(xlib):
    r = np.random.default_rng(6)
    for n in (0, 1, 2, 9, 33, 100):
        a = r.standard_normal(n).astype(np.float32)
        for K in (1, 3, 64):
            want, got, _, _ = composed(xlib, a, a.astype(np.float64), K, [8, 4])
            assert same(want, got), (n, K)
    n = 4000
    for bad in (np.nan, np.inf, -np.inf):
        a = r.standard_normal(n).astype(np.float32)
        a[n // 2] = bad
        want, got, _, _ = composed(xlib, a, np.ones(n), 256, [8, 4, 8])
        assert same(want, got) or (np.isnan(want) and np.isnan(got)), bad


def test_composed_walk_is_short(xlib):
    """At the append kernel's shape (10^6 rows, 38,912 chunks) the final walk
    takes almost every composite as it is: a sum of squares descends a handful
    of times, a signed dot product a few dozen."""
    r = np.random.default_rng(7)
    n = 1_000_000
    q = r.standard_normal(n).astype(np.float32)
    v = r.standard_normal(n)
    want, got, redone, desc = composed(xlib, q, v, 38912, [8, 4, 8, 16])
    assert same(want, got)
    assert redone <= 40 and desc <= 80, (redone, desc)
    want, got, redone, desc = composed(xlib, v.astype(np.float32), v, 38912, [8, 4, 8, 16])
    assert same(want, got)
    assert redone <= 4 and desc <= 8, (redone, desc)


def kernel_levels(lib, a, b, K, rb):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float64)
    fp = ctypes.POINTER(ctypes.c_float)
    dp = ctypes.POINTER(ctypes.c_double)
    re, de = ctypes.c_int(0), ctypes.c_int(0)
    got = getattr(lib, "xc_host_kernel%d" % rb)(a.ctypes.data_as(fp), b.ctypes.data_as(dp),
                                                 a.size, K, ctypes.byref(re), ctypes.byref(de))
    return got, re.value, de.value


@pytest.mark.parametrize("K", [1, 64, 1000, 8192])
def test_kernel_levels_equal_sequential(xlib, K):
    """The append kernel's own levels (4-residue chunk, sub-group and warp
    records, 8-residue block and group records whose group lanes give up where
    a block cannot vouch) give the sequential chain bit for bit."""
    r = np.random.default_rng(K + 11)
    for name, a, b in cases(K):
        bd = b.astype(np.float64)
        if name in ("signed", "wide"):
            bd = bd * (1.0 + 2.0 ** -30 * r.standard_normal(bd.size))
        want = xlib.xc_host_sequential_d(a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                         np.ascontiguousarray(bd).ctypes.data_as(
                                             ctypes.POINTER(ctypes.c_double)), a.size)
        for rb in (4, 8):
            got, _, _ = kernel_levels(xlib, a, bd, K, rb)
            assert same(want, got) or (np.isnan(want) and np.isnan(got)), (name, K, rb)


def test_block_residues_shorten_the_walk(xlib):
    """Signed dot products at 10^6 rows in the kernel's shape (256 blocks of
    256 chunks): 8 residues at the block and group levels let the walk cross
    blocks that 4 would descend into."""
    r = np.random.default_rng(12)
    n, K = 1_000_000, 256 * 256
    tot = {4: 0, 8: 0}
    for it in range(4):
        q = r.standard_normal(n).astype(np.float32)
        v = r.standard_normal(n) * (1.0 + it)
        v -= q.astype(np.float64) * (q.astype(np.float64) @ v) / float(q.astype(np.float64) @ q)
        want = xlib.xc_host_sequential_d(q.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                         v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n)
        for rb in (4, 8):
            got, _, desc = kernel_levels(xlib, q, v, K, rb)
            assert same(want, got), (it, rb)
            tot[rb] += desc
    assert tot[8] < tot[4], tot


def test_translation_is_used(xlib):
    """The checks must not reject everything: with guesses a few ulps off, chunks of
    squares, of positive terms and of rounding ties are resolved by translation."""
    for name, a, b in cases(5):
        if name not in ("squares", "positive", "ties"):
            continue
        for k in (0.0, 1.0, 2.0, 3.0, -5.0):
            want, got, redone = run(xlib, a, b, 64, 2, k)
            assert same(want, got), (name, k)
            assert redone <= 2, (name, k, redone)


def test_random_sweep(xlib):
    r = np.random.default_rng(4)
    for it in range(200):
        n = int(r.integers(0, 3000))
        scale_a = 2.0 ** int(r.integers(-20, 20))
        a = (r.standard_normal(n) * scale_a).astype(np.float32)
        if it % 3 == 0:
            b = a
        elif it % 3 == 1:
            b = np.abs(r.standard_normal(n)).astype(np.float32)
        else:
            b = (r.integers(-3, 4, n) / 2).astype(np.float32)
        K = int(r.integers(1, 300))
        want, got, _ = run(xlib, a, b, K)
        assert same(want, got), (it, n, K)


def _hinge_lib(xlib):
    fp = ctypes.POINTER(ctypes.c_float)
    dp = ctypes.POINTER(ctypes.c_double)
    xlib.xh_host_sequential.restype = None
    xlib.xh_host_sequential.argtypes = [fp, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    xlib.xh_host_chunked.restype = None
    xlib.xh_host_chunked.argtypes = [fp, fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, dp, ctypes.POINTER(ctypes.c_int)]
    return xlib


def run_hinge(lib, b, y, x, head, min_span, K):
    b, y, x = (np.ascontiguousarray(v, np.float32) for v in (b, y, x))
    tail = b.size
    ng = (tail - 1 - (head + 1)) // min_span + 1 if tail - 1 >= head + 1 else 0
    want = np.full(3 * max(ng, 1), -7.0)
    got = np.full(3 * max(ng, 1), -7.0)
    dp = ctypes.POINTER(ctypes.c_double)
    lib.xh_host_sequential(_ptr(b), _ptr(y), _ptr(x), tail, head, min_span,
                           want.ctypes.data_as(dp))
    re = ctypes.c_int(0)
    lib.xh_host_chunked(_ptr(b), _ptr(y), _ptr(x), tail, head, min_span, K,
                        got.ctypes.data_as(dp), ctypes.byref(re))
    return want, got, re.value


def hinge_cases(seed):
    r = np.random.default_rng(seed)
    n = 30000
    x = np.sort(r.standard_normal(n).astype(np.float32))[::-1].copy()
    y = r.standard_normal(n).astype(np.float32)
    b = np.maximum(r.standard_normal(n), 0).astype(np.float32)
    yield "hinge parent", b, y, x
    yield "intercept, skewed y", np.ones(n, np.float32), (y + 0.3).astype(np.float32), x
    xq = np.sort((r.integers(0, 50, n) / 8).astype(np.float32))[::-1].copy()  # ties: d = 0
    yield "quantised x", np.abs(y), (r.integers(-4, 5, n) / 4).astype(np.float32), xq
    b2 = b.copy()
    b2[n // 3: n // 2] = 0  # a run of zero parent values
    yield "zero run", b2, y, x
    yield "wide", (np.abs(y) * 2.0 ** r.integers(-30, 30, n)).astype(np.float32), y, x


@pytest.mark.parametrize("K", [1, 2, 32, 96, 256, 512])
def test_hinge_scalars_chunked_equal_sequential(xlib, K):
    lib = _hinge_lib(xlib)
    for name, b, y, x in hinge_cases(6):
        for head, span in ((0, 1), (3, 7), (100, 33)):
            want, got, _ = run_hinge(lib, b, y, x, head, span, K)
            assert (want.view(np.uint64) == got.view(np.uint64)).all(), (name, K, head, span)


def test_hinge_scalars_few_chunks_redone(xlib):
    lib = _hinge_lib(xlib)
    r = np.random.default_rng(7)
    n = 200000
    x = np.sort(r.standard_normal(n).astype(np.float32))[::-1].copy()
    b = np.maximum(r.standard_normal(n), 0).astype(np.float32)
    y = (r.standard_normal(n) + 0.1).astype(np.float32)
    want, got, redone = run_hinge(lib, b, y, x, 0, 6, 256)
    assert (want.view(np.uint64) == got.view(np.uint64)).all()
    # six chains walked over 255 chunks each
    assert redone <= 0.1 * 6 * 255, redone


def test_hinge_scalars_short_and_empty_chunks(xlib):
    lib = _hinge_lib(xlib)
    r = np.random.default_rng(8)
    for tail in (1, 2, 3, 5, 31, 33, 40):
        x = np.sort(r.standard_normal(tail).astype(np.float32))[::-1].copy()
        y = r.standard_normal(tail).astype(np.float32)
        b = np.abs(r.standard_normal(tail)).astype(np.float32)
        for K in (32, 64):
            for head, span in ((0, 1), (1, 2)):
                want, got, _ = run_hinge(lib, b, y, x, head, span, K)
                assert (want.view(np.uint64) == got.view(np.uint64)).all(), (tail, K, head)


def test_zero_prefix_needs_no_rerun(xlib):
    """A hinge parent is zero on one side of its knot: every chain then stays at
    +0 for a stretch of chunks, which the run from +0 resolves."""
    lib = _hinge_lib(xlib)
    r = np.random.default_rng(9)
    n = 100000
    x = np.sort(r.standard_normal(n).astype(np.float32))[::-1].copy()
    y = r.standard_normal(n).astype(np.float32)
    b = np.maximum(r.standard_normal(n), 0).astype(np.float32)
    b[: n // 2] = 0
    want, got, redone = run_hinge(lib, b, y, x, 0, 5, 256)
    assert (want.view(np.uint64) == got.view(np.uint64)).all()
    assert redone <= 60, redone
    z = r.standard_normal(n).astype(np.float32)
    z[: n // 3] = 0
    want, got, redone = run(xlib, z, z, 512)
    assert same(want, got)
    assert redone <= 4, redone


def test_kernel_levels_on_a_fits_appends(xlib):
    """The Gram-Schmidt chains of the first appends of the hinge-search fit
    (10^5 rows x 20 inputs; the reference's golden term path: hinge columns
    that are zero on most rows, their products with parents, in the append
    kernel's 49 blocks)
    through the kernel's levels give the sequential chains bit for bit."""
    import json

    from mars_gb300 import workloads

    X, _y, _kw = workloads.hinge_search()
    with open(os.path.join(HERE, "golden", "hinge_search.json")) as f:
        model = json.load(f)["model"]
    n = X.shape[0]
    K = min(256, -(-n // (256 * 8))) * 256
    s = 1.0 / np.sqrt((X.astype(np.float64) ** 2).mean(0))
    b0 = (np.ones(n) / np.sqrt(n)).astype(np.float32)
    B, Q = [b0], [b0]
    fp = ctypes.POINTER(ctypes.c_float)
    dp = ctypes.POINTER(ctypes.c_double)
    chains = 0
    for t in model[1:9]:
        xp, bp, sx = X[:, t["input"]], B[t["basis"]], np.float32(s[t["input"]])
        h = np.float32(t["hinge"]) if t["hinge"] is not None else None
        if t["type"] == "l":
            val = (sx * bp) * xp
        elif t["type"] == "+":
            val = (sx * bp) * np.maximum(xp - h, np.float32(0))
        else:
            val = (sx * bp) * np.maximum(h - xp, np.float32(0))
        v = val.astype(np.float64)
        for q in [val] + Q:
            want = xlib.xc_host_sequential_d(q.ctypes.data_as(fp), v.ctypes.data_as(dp), n)
            got, _, _ = kernel_levels(xlib, q, v, K, 8)
            assert same(want, got), (t, chains)
            chains += 1
            if q is not val:
                v = v - float(q.astype(np.float64) @ v) * q.astype(np.float64)
        B.append((val / np.float32(np.sqrt(np.sum(val.astype(np.float64) ** 2)))).astype(
            np.float32))
        Q.append((v / np.sqrt(v @ v)).astype(np.float32))
    assert chains == sum(1 + k for k in range(1, 9))
