"""bench.py's multi-rank host logic on CPU (gloo, world size 2).

The forward pass of one fit does not shard: `bench.py --gpus N` runs N replicas,
one per rank, and reports the max over ranks of the timed span and the sum of
their work. These tests run that reduction over two gloo ranks, and the
reference arm under torchrun with two ranks (rank 0 alone times it and prints).
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


REDUCE = r"""
import bench
t = bench.dist()
rank = int(__import__("os").environ["RANK"])
print(bench.allmax(t, 1.5 + rank), bench.allsum(t, 10 * (rank + 1)))
t.destroy_process_group()
"""


def test_replica_reductions_over_gloo():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", REDUCE], cwd=ROOT, env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True))
    outs = [p.communicate(timeout=300) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err
        mx, total = out.split()
        assert float(mx) == 2.5  # the slowest rank's span
        assert float(total) == 30.0  # the work of both replicas


def test_reference_arm_under_torchrun_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3",
           "--workload", "plain_fit"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1  # rank 0 only
    line = lines[0]
    assert line["impl"] == "reference"
    # plain_fit is a linear-only fit: no knots are scored, the time is what is measured
    assert line["ms_per_step"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["steps"] == 1 and line["warmup"] == 3


def test_reference_arm_epoch_steps():
    """The epoch-step reference arm (the default workload's): each step one
    eval of a sample of an epoch's candidates on the reference fit's basis
    replayed from its fixture; here on the small case of the same shape."""
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--steps", "2", "--warmup", "3",
           "--workload", "precision_stress_small"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] == 3
    assert line["cpu_baseline"]["kind"] == "port"


def test_epoch_sample_replays_the_reference_basis():
    """The sampled state is the reference fit's basis at that epoch: its
    column count follows the term path, and each sampled candidate obeys the
    degree and self-interaction rules."""
    import bench
    from tests.golden import cases

    X, y, w, kw = cases.fit_case("precision_stress_small")
    path = bench.reference_path("precision_stress_small")
    state = {}
    dt, kn = bench.cpu_epoch_sample(X, y, kw, path, 3, state, 2, ncols=4, nparents=2)
    assert dt > 0 and kn > 0
    assert state["epochs"] == 3
    m = state["algo"].nbasis()
    assert 1 + 3 <= m <= 1 + 6
    assert bench.path_epochs(path) >= 3


def test_orth_by_step_follows_the_epochs():
    """The per-step orthogonality report picks, for each epoch, the entry of
    the leading basis that epoch reached (a linear term adds one column, a
    hinge pair two, a rejected column none)."""
    import numpy as np

    import bench

    class Fake:
        def orth_error_by_terms(self):
            return np.arange(1, 8) * 1e-9, 1.0 - np.arange(1, 8) * 0.1

    out = bench.orth_by_step(Fake(), [3, 5, 5, 6, 7])
    assert out["terms"] == [3, 5, 5, 6, 7]
    assert out["max_abs_QtQ_minus_I"] == pytest.approx([3e-9, 5e-9, 5e-9, 6e-9, 7e-9])
    assert out["rss"] == pytest.approx([0.7, 0.5, 0.5, 0.4, 0.3])
    assert bench.orth_by_step(Fake(), []) == {"terms": [], "max_abs_QtQ_minus_I": [], "rss": []}
