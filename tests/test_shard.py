"""One fit sharded by input column over several ranks (mars_gb300/shard.py).

Each rank evaluates only its block of input columns, the (linear, hinge, cut)
rows are all-gathered, and every rank appends the same term. Run here as two
and three gloo ranks on CPU with the oracle (the C restatement of the
reference CPU path) as each rank's evaluator: every rank must reach the
reference's own term path on the golden fits, the same one a single process
reaches.
"""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_owned_columns_partition():
    from mars_gb300.shard import owned_columns

    for p in (1, 2, 5, 20, 101):
        for world in (1, 2, 3, 8):
            blocks = [owned_columns(p, r, world) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == p
            assert all(a[1] == b[0] for a, b in zip(blocks, blocks[1:]))
            assert all(hi >= lo for lo, hi in blocks)  # a rank may own nothing


def test_combine_takes_each_entry_from_its_owner():
    from mars_gb300.shard import combine

    rng = np.random.default_rng(0)
    p, m = 5, 3
    lin, hin = rng.random((p, m)), rng.random((p, m))
    cut = np.where(rng.random((p, m)) < 0.3, np.nan, rng.standard_normal((p, m)))
    cut[0, 0] = -0.0
    parts = [(0, 2, lin[:2], hin[:2], cut[:2]), (2, 2, lin[2:2], hin[2:2], cut[2:2]),
             (2, 5, lin[2:], hin[2:], cut[2:])]
    L, H, C = combine(parts, p)
    assert L.tobytes() == lin.tobytes() and H.tobytes() == hin.tobytes()
    assert C.tobytes() == cut.tobytes()  # bit for bit, -0.0 and NaN included
    # the first maximum in row-major order: the lowest (input, parent) on a tie
    L[1, 2] = L[3, 0] = 10.0
    assert np.unravel_index(np.argmax(L), L.shape) == (1, 2)


RANK_FIT = r"""
import json, os, sys
import torch.distributed as dist
sys.path.insert(0, os.getcwd())
import oracle
from mars_gb300.mars import forward_pass
from mars_gb300.shard import sharded
from tests.golden import cases
dist.init_process_group("gloo")
out = {}
for name in sys.argv[1:]:
    X, y, w, kw = cases.fit_case(name)
    model = forward_pass(sharded(oracle.marslib_for("port")), X, y, w, threads=1, **kw)
    out[name] = [(r["type"].decode(), int(r["basis"]), int(r["input"]),
                  None if r["hinge"] != r["hinge"] else float(r["hinge"])) for r in model]
print("RESULT " + json.dumps(out))
dist.destroy_process_group()
"""


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_fit_reaches_the_reference_term_path(world, port):
    names = ["hinge_search_small", "precision_stress_small", "fastmars_caps", "weighted_nan"]
    addr = _free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(addr))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_FIT] + names, cwd=ROOT,
                                      env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True))
    outs = [p.communicate(timeout=600) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err[-3000:]
        got = json.loads(out.split("RESULT ", 1)[1])
        for name in names:
            with open(os.path.join(ROOT, "tests", "golden", name + ".json")) as f:
                want = [(r["type"], r["basis"], r["input"], r["hinge"])
                        for r in json.load(f)["model"]]
            assert [tuple(r) for r in got[name]] == want, name
