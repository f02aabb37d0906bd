#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own ``mars.py`` over its own ``marslib`` binding, built
from the reference sources by ``make -C oracle ref`` into ``oracle/_ref/``.
This needs the reference checkout, named by MARS_REFERENCE_DIR; the fixtures it writes are small JSON/npz files that the
tests read anywhere, with no access to the reference.

Each term-path fixture stores, per fitted basis row: type, parent basis,
input column, hinge cut, r2, r2_cv, order; plus a sha256 of the generated
inputs so a test can tell a generator change from a parity failure.

    python tests/golden/make_golden.py            # all fixtures
    python tests/golden/make_golden.py plain_fit  # one
"""
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("MARS_REFERENCE_DIR")
sys.path.insert(0, ROOT)

from mars_gb300 import workloads  # noqa: E402
from tests.golden import cases  # noqa: E402


def _import_reference():
    if not REF or not os.path.isfile(os.path.join(REF, "mars.py")):
        raise SystemExit("set MARS_REFERENCE_DIR to the reference checkout")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + REF],
                   check=True, capture_output=True)
    sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
    sys.path.insert(0, REF)
    import mars as ref_mars  # noqa: E402  (reference mars.py)
    import marslib as ref_marslib  # noqa: E402  (reference binding)
    assert os.path.dirname(os.path.abspath(ref_mars.__file__)) == os.path.abspath(REF)
    return ref_mars, ref_marslib


def model_rows(model):
    rows = []
    for r in model:
        rows.append({
            "type": r["type"].decode(),
            "basis": int(r["basis"]),
            "input": int(r["input"]),
            "hinge": None if np.isnan(r["hinge"]) else float(r["hinge"]),
            "r2": float(r["r2"]),
            "r2_cv": float(r["r2_cv"]),
            "order": int(r["order"]),
        })
    return rows


def fit_fixture(ref_mars, name):
    X, y, w, kw = cases.fit_case(name)
    t0 = time.time()
    model = ref_mars.fit(X, y, w, threads=-1, **kw)
    dt = time.time() - t0
    out = {
        "case": name,
        "kwargs": {k: v for k, v in kw.items()},
        "shape": list(X.shape),
        "digest": workloads.digest(X, y) if w is None else workloads.digest(X, y, w),
        "model": model_rows(model),
        "reference_seconds": round(dt, 3),
        "threads": os.cpu_count(),
    }
    path = os.path.join(HERE, name + ".json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("%-24s %3d terms  %.2fs" % (name, len(model), dt))


def eval_fixture(ref_marslib, name):
    X, y, w, appends, evals = cases.eval_case(name)
    algo = ref_marslib.MarsAlgo(X, y, w, cases.EVAL_MAX_TERMS)
    mses = [algo.append(t, xc, bc, h) for (t, xc, bc, h) in appends]
    res = {"yvar": algo.yvar(), "mses": np.array(mses), "nbasis": algo.nbasis()}
    for i, (min_span, endspan, linear_only) in enumerate(evals):
        m = algo.nbasis()
        mask = cases.eval_mask(X.shape[1], m, i)
        d, lin, hin, cut = algo.eval(mask, min_span, endspan, linear_only, 1)
        res["dsse_%d" % i] = np.array(d)
        res["lin_%d" % i] = lin
        res["hin_%d" % i] = hin
        res["cut_%d" % i] = cut
    res["digest"] = np.array(workloads.digest(X, y, w))
    np.savez(os.path.join(HERE, name + ".npz"), **res)
    print("%-24s eval fixture (%d evals)" % (name, len(evals)))


def prune_fixture(ref_mars, name):
    """The reference's prune (mars.py:622-695) on the expanded golden model
    of a fit case, or on the small scenarios."""
    res = {}
    if name == "prune_scenarios":
        for i, (B, y, w, kw) in enumerate(cases.prune_scenarios()):
            res["beta_%d" % i] = ref_mars.prune(B, y, w, **kw)
        res["digest"] = np.array(workloads.digest(
            *[a for B, y, w, _ in cases.prune_scenarios() for a in (B, y)]))
    else:
        fit = name[len("prune_"):]
        with open(os.path.join(HERE, fit + ".json")) as f:
            rows = json.load(f)["model"]
        X, y, w, _ = cases.fit_case(fit)
        model = cases.model_from_rows(rows)
        B = ref_mars.expand(X, model)
        for tag, kw in cases.prune_variants(len(model)):
            res["beta_" + tag] = ref_mars.prune(B, y, w, **kw)
        res["digest"] = np.array(workloads.digest(B, y))
    np.savez(os.path.join(HERE, name + ".npz"), **res)
    print("%-24s prune fixture" % name)


def main(argv):
    ref_mars, ref_marslib = _import_reference()
    names = argv or (cases.FIT_CASES + cases.EVAL_CASES + cases.PRUNE_CASES)
    for name in names:
        if name in cases.FIT_CASES:
            fit_fixture(ref_mars, name)
        elif name in cases.PRUNE_CASES:
            prune_fixture(ref_mars, name)
        else:
            eval_fixture(ref_marslib, name)


if __name__ == "__main__":
    main(sys.argv[1:])
