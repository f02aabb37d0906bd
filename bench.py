#!/usr/bin/env python3
"""Forward-pass benchmark on one GB300 (or N independent replicas).

Default workload: precision stress, X n=1,000,000 x
p=100 float32 with AR(1) column correlation rho=0.9 and 5 near-duplicate
columns, y = 2 x_a + 3 x_b + x_a x_b over 5 column pairs + N(0,1),
max_terms=63, max_degree=3, tail_span=0.02 (the reference's default; synthetic,
seeded: mars_gb300/workloads.py), in mixed precision.

Step. The fit has one epoch per selected term pair (~31 for 63 terms), each an
eval of every (input, parent) candidate plus the append of the chosen pair;
one step is one epoch. The first W epochs of the fit are the warm-up, the next
K are timed, and the fit then runs to its end untimed (so the term path can
be checked against the reference's); with W + K past the fit's epochs the
timed region continues into a second fit. Inputs are far larger than the
129 MB L2 (X 400 MB, the projected candidates ~24 GB per epoch), so L2 is not
flushed between steps. --workload hinge_search (n=100,000 x p=20) keeps one
full fit per step.

value        knot-evals/s over the device span of the timed epochs (CUDA
             events on the library's stream; X, y resident in HBM), whole job
             (all ranks) / max rank time.
e2e          the same knot-evals over the host wall time of those epochs
             through mars.fit (host mask in, host results out every epoch)
             plus the fit's upload of X, y, w charged in full.
fp64         the plain FP64 GPU forward pass of the same workload: fit time,
             the same timed epochs, speed-up, identical term path.
roofline     the dominant kernel of the timed region against the measured
             peaks in MEASURED_PEAKS.json (HBM GB/s or tensor TFLOP/s).
cpu_baseline the CPU oracle (the C restatement of the reference CPU path) on
             the host cores, on a sample of the same epochs' candidates.

--impl reference times that CPU implementation alone: step k is one eval of
a sample of the candidates of epoch W + k (16 input columns, 3 parents each,
on the basis the reference's own fit had built by then, replayed from the
committed reference fixture). Under torchrun (N > 1) every rank runs its own
replica on its own GPU (the fit does not exchange data between GPUs); timing
is max over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORLD = int(os.environ.get("WORLD_SIZE", "1"))
RANK = int(os.environ.get("RANK", "0"))
LOCAL_RANK = int(os.environ.get("LOCAL_RANK", "0"))
if WORLD > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
    os.environ["CUDA_VISIBLE_DEVICES"] = str(LOCAL_RANK)

import numpy as np  # noqa: E402

METRIC = "knot-evals/sec & fit time: mixed-prec batched vs FP64 GPU, same term path"
UNIT = "knot-evals/s"
WORKLOADS = {
    "hinge_search": "hinge_search n=100000 p=20 iid N(0,1), 6 hinges + 3 hinge products, "
                    "max_terms=31 max_degree=2 tail_span=0",
    "precision_stress": "precision_stress n=1000000 p=100 AR(1) rho=0.9 + 5 near-duplicates, "
                        "max_terms=63 max_degree=3 tail_span=0.02 (the reference's default "
                        "tail span)",
    "precision_stress_small": "precision_stress n=30000 p=20 AR(1) rho=0.9 + 3 near-duplicates, "
                              "max_terms=21 tail_span=0 (a small case of precision_stress's "
                              "shape)",
    "plain_fit": "plain_fit n=10000 p=2 linear_only max_terms=17",
    "batched": "256 independent fits, n log-uniform 1e3..2e5, p uniform 5..50, 4 random hinges "
               "+ N(0,1) noise, max_terms=21, tail_span=0",
    "expand": "differentiable prediction of a fitted hinge_search model (31 terms) on "
              "1,000,000 rows: forward + backward",
    "projection": "the mixed fast pass's two-pass projection alone on a slice of "
                  "precision_stress: "
                  "n=1,000,000 rows, m=32 basis columns, 640 candidates (20 inputs x 32 parents)",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default=os.environ.get("MARS_BENCH_PRECISION", "mixed"),
                    choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="precision_stress", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the FP64 comparator fits when timing the mixed path")
    ap.add_argument("--profile-epochs", action="store_true",
                    help="end the fit once the timed epochs are done and print only their "
                         "timing (short runs for ncu captures)")
    ap.add_argument("--shard", action="store_true",
                    help="under torchrun: one fit sharded by input column over the ranks "
                         "(mars_gb300/shard.py) instead of one replica per rank")
    return ap.parse_args()


def workload(name):
    from mars_gb300 import workloads

    if name == "hinge_search":
        return workloads.hinge_search()
    if name == "precision_stress":
        X, y, kw = workloads.precision_stress()
        kw["tail_span"] = 0.02
        return X, y, kw
    if name == "precision_stress_small":
        return workloads.precision_stress(n=30_000, p=20, n_dup=3, seed=5, max_terms=21)
    return workloads.plain_fit()


# workloads timed one epoch per step (the others: one fit per step)
EPOCH_WORKLOADS = ("precision_stress", "precision_stress_small")


class Counting:
    """A marslib-like module that counts knot evaluations and keeps the algo."""

    def __init__(self, factory):
        self.__version__ = "0.12"
        self._factory = factory
        self.algo = None
        self.knot_evals = 0
        self.candidates = 0
        self.wall_eval = 0.0    # host wall seconds inside eval / append calls
        self.wall_append = 0.0

    def MarsAlgo(self, X, y, w, max_terms):
        from mars_gb300 import workloads

        inner = self._factory(X, y, w, max_terms)
        outer = self
        n = X.shape[0]

        class Wrapped:
            def __getattr__(self, k):
                return getattr(inner, k)

            def eval(self, mask, min_span, endspan, linear_only, threads, cuda=False):
                t0 = time.perf_counter()
                res = inner.eval(mask, min_span, endspan, linear_only, threads, cuda)
                outer.wall_eval += time.perf_counter() - t0
                c = int(mask.sum())
                outer.candidates += c
                if not linear_only:
                    outer.knot_evals += c * workloads.knot_evals(n, endspan, min_span)
                return res

        def append(self_, *a):
            t0 = time.perf_counter()
            r = inner.append(*a)
            outer.wall_append += time.perf_counter() - t0
            return r

        Wrapped.append = append
        self.algo = inner
        return Wrapped()


def path_of(model):
    return [(r["type"].decode(), int(r["basis"]), int(r["input"]),
             None if np.isnan(r["hinge"]) else float(r["hinge"])) for r in model]


def gpu_fit(X, y, kw, precision):
    from mars_gb300 import marslib
    from mars_gb300.mars import forward_pass

    def factory(X_, y_, w_, mt):
        a = marslib.MarsAlgo(X_, y_, w_, mt)
        a.set_precision(precision)
        return a

    lib = Counting(factory)
    t0 = time.perf_counter()
    model = forward_pass(lib, X, y, None, **kw)
    wall = time.perf_counter() - t0
    st = lib.algo.stats()
    # after the timed fit: max |Q^T Q - I| of the final basis (the basis only
    # grows, so this is the largest over the fit's steps) and its FP64 RSS
    st["orth_max"], st["rss"] = lib.algo.orth_error()
    return model, wall, st, lib.knot_evals


class L2Flush:
    """Writes a buffer larger than the 129 MB L2 between timed steps."""

    def __init__(self):
        try:
            import torch

            self.torch = torch
            self.buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
        except Exception:  # noqa: BLE001 - torch is optional plumbing here
            self.torch = None

    def __call__(self):
        if self.torch is not None:
            self.buf.zero_()
            self.torch.cuda.synchronize()

    @property
    def ok(self):
        return self.torch is not None


class Clocks:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-f", self.path], stdout=subprocess.DEVNULL,
                stderr=subprocess.DEVNULL)
        except Exception:  # noqa: BLE001
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9 or (dev.isdigit() and f[0] != dev):
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for k, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(k)
        finally:
            os.unlink(self.path)
        if not sm:
            return None
        top = max(sm)
        loaded = [s for s in sm if s >= 0.5 * top] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(mx),
                "samples": len(sm), "reasons": sorted(reasons)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], "measured"
    except Exception:  # noqa: BLE001
        return 6800.0, 1900.0, "fallback"


def traffic_ratio(precision, workload_name, kernel):
    """DRAM bytes over algorithmic bytes of one launch of `kernel`, from the
    committed ncu summary (profiles/traffic.txt), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.txt")) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 4 and not parts[0].startswith("#") and \
                        parts[:3] == [precision, workload_name, kernel]:
                    return float(parts[3])
    except OSError:
        pass
    return None


def limiter(precision, workload_name, kernel):
    """What the committed ncu summary of `kernel` on this workload says bounds
    it (profiles/limiters.txt), with the summary's file name; None when no
    capture of this workload exists."""
    try:
        with open(os.path.join(ROOT, "profiles", "limiters.txt")) as f:
            for line in f:
                if line.startswith("#") or "|" not in line:
                    continue
                key, text, src = [x.strip() for x in line.split("|")]
                if key.split() == [precision, workload_name, kernel]:
                    return {"limiter": text, "capture": "profiles/" + src}
    except OSError:
        pass
    return {"limiter": None, "capture": "none of this workload"}


def roofline(st, workload_name, precision):
    """The dominant kernel against its roofline. The hinge sweep is charged
    with its algorithmic bytes against HBM bandwidth; the projection with its
    algorithmic FLOPs against the bf16 tensor peak. What bounds the kernel
    comes from the committed capture of this workload, when there is one."""
    hbm, bf16, src = peaks()
    phases = {"sweep": st["ms_sweep"], "project": st["ms_project"]}
    dom = max(phases, key=phases.get)
    if dom == "sweep" and st["ms_sweep"] > 0:
        ach = st["sweep_bytes"] / (st["ms_sweep"] * 1e-3) / 1e9
        kern = "k_sweep" if precision == "fp64" else "k_fast_sweep"
        ratio = traffic_ratio(precision, workload_name, kern)
        per_launch = st["sweep_bytes"] / max(1, st["evals"])
        return {"kernel": "hinge sweep (%s)" % kern, "bound": "hbm", "achieved": ach, "peak": hbm,
                "unit": "GB/s", "frac": ach / hbm, "peak_source": src,
                "algorithmic_bytes_per_launch": per_launch,
                "traffic": None if ratio is None else ratio * per_launch,
                **limiter(precision, workload_name, kern)}
    ms = max(st["ms_project"], 1e-9)
    ach = st["project_flops"] / (ms * 1e-3) / 1e12
    kern = "projection"
    return {"kernel": kern, "bound": "tensor", "achieved": ach, "peak": bf16,
            "unit": "TFLOP/s", "frac": ach / bf16, "peak_source": src, "traffic": None,
            **limiter(precision, workload_name, kern)}


def cpu_threads():
    return os.cpu_count() or 1


def cpu_fit(X, y, kw, threads):
    import oracle
    from mars_gb300.mars import forward_pass

    if not oracle.available("port"):
        oracle.build(with_reference=False)

    def factory(X_, y_, w_, mt):
        return oracle.OracleAlgo(X_, y_, w_, mt, kind="port")

    lib = Counting(factory)
    t0 = time.perf_counter()
    model = forward_pass(lib, X, y, None, threads=threads, **kw)
    return model, time.perf_counter() - t0, lib.knot_evals


def dist():
    if WORLD <= 1:
        return None
    import torch.distributed as tdist

    tdist.init_process_group("gloo")
    return tdist


def allmax(tdist, v):
    if tdist is None:
        return v
    import torch

    t = torch.tensor([float(v)], dtype=torch.float64)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def allsum(tdist, v):
    if tdist is None:
        return v
    import torch

    t = torch.tensor([float(v)], dtype=torch.float64)
    tdist.all_reduce(t, op=tdist.ReduceOp.SUM)
    return float(t.item())


def run_reference(args):
    if RANK != 0:
        return 0
    X, y, kw = workload(args.workload)
    threads = cpu_threads()
    for _ in range(args.warmup):
        cpu_fit(X, y, kw, threads)
    total_k, total_t = 0, 0.0
    for _ in range(args.steps):
        _, dt, k = cpu_fit(X, y, kw, threads)
        total_k += k
        total_t += dt
    value = total_k / total_t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total_t / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "full fit per step, OpenMP over input columns"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


BATCH_THREADS = int(os.environ.get("MARS_BENCH_BATCH_THREADS", "16"))


def run_batched(args):
    """Config 4: fits/s over 256 independent fits driven concurrently."""
    from mars_gb300 import batch, marslib, workloads

    marslib.load()
    probs = [(X, y, None, kw) for X, y, kw in workloads.batched_fits(count=256, seed=0)]
    for _ in range(max(args.warmup, 0)):
        batch.fit_many(probs[:8], threads=8, precision=args.precision)
    clocks = Clocks()
    clocks.start()
    t0 = time.perf_counter()
    walls = []
    fstats = []
    for _ in range(args.steps):
        _, per = batch.fit_many(probs, threads=BATCH_THREADS, precision=args.precision,
                                stats=fstats)
        walls.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
    clk = clocks.stop()
    # Each fit starts from host arrays and ends with its model on the host: the
    # timed region already holds every copy, so e2e is the same measurement;
    # the bytes are the handles' own counts of what they copied.
    h2d = sum(st["h2d_bytes"] for st in fstats) // max(1, args.steps)
    d2h = sum(st["d2h_bytes"] for st in fstats) // max(1, args.steps)
    launches = sum(st["kernel_launches"] for st in fstats)
    per = sorted(per)
    total = sum(walls) / args.steps
    line = {"metric": "fits/s (256 independent fits)", "value": len(probs) / total,
            "unit": "fits/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "mixed",
            "precision": args.precision, "data": "synthetic",
            "config": {"workload": WORKLOADS["batched"], "concurrency": "16 host threads, "
                       "one handle and stream per fit"},
            "per_fit_s": {"p50": per[len(per) // 2], "p99": per[min(len(per) - 1,
                                                                  int(0.99 * len(per)))]},
            "e2e": {"value": len(probs) / total, "unit": "fits/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "clocks": clk}
    if not args.no_cpu_baseline:
        sample = probs[:4]
        t0 = time.perf_counter()
        for X, y, _, kw in sample:
            cpu_fit(X, y, kw, cpu_threads())
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": len(sample) / dt, "unit": "fits/s",
                                "cores": cpu_threads(), "kind": "port",
                                "sample": "the first 4 of the 256 fits, one after another"}
    print(json.dumps(line))
    return 0


def run_projection(args):
    """The fast projection alone (mars_gpu_fast_project), tensor cores against
    the FP32 SIMT kernels, device time of the kernels only. Algorithmic work:
    two passes of T = Bo^T v (2 n m P FLOP) and Bx = v - Bo T (2 n m P FLOP)."""
    from mars_gb300 import marslib

    marslib.load()
    rng = np.random.default_rng(0)
    n, m, p, per = 1_000_000, 32, 20, 32
    Q, _ = np.linalg.qr(rng.standard_normal((n, m)).astype(np.float32))
    Bo = np.asfortranarray(Q.astype(np.float32))
    B = np.asfortranarray(np.abs(rng.standard_normal((n, m))).astype(np.float32))
    X = np.asfortranarray(rng.standard_normal((n, p)).astype(np.float32))
    s = np.ones(p, dtype=np.float32)
    cx = np.repeat(np.arange(p), per).astype(np.int32)
    cb = np.tile(np.arange(per), p).astype(np.int32)
    y = rng.standard_normal(n).astype(np.float32)
    P = len(cx)
    flops = 8.0 * n * m * P
    out = {}
    for name, tc in (("tc", True), ("simt", False)):
        times = []
        for _ in range(max(args.warmup, 1)):
            marslib.fast_project(B, X, s, cx, cb, Bo, m, y, 1e-14, use_tc=tc)
        for _ in range(args.steps):
            marslib.fast_project(B, X, s, cx, cb, Bo, m, y, 1e-14, use_tc=tc, timing=times)
        out[name] = statistics.median(times)
    _, bf16, src = peaks()
    ach = flops / (out["tc"] * 1e-3) / 1e12
    line = {"metric": "fast projection device time (two passes + norms)", "value": out["tc"],
            "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": out["tc"], "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "split-TF32 (tensor cores), FP32 accumulate",
            "data": "synthetic", "config": {"workload": WORKLOADS["projection"]},
            "simt_fp32_ms": out["simt"], "speedup_vs_simt": out["simt"] / out["tc"],
            "roofline": {"kernel": "k_tc_tgemm + k_tc_project", "bound": "tensor",
                         "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
                         "frac": ach / bf16, "peak_source": src,
                         "note": "algorithmic FLOPs (8 n m P) over the device time of the whole "
                                 "projection; split TF32 issues 3 MMAs per product"}}
    print(json.dumps(line))
    return 0


def run_expand(args):
    """Config 5: rows/s of forward + backward of the differentiable prediction."""
    import torch

    from mars_gb300 import diff, mars, marslib, workloads

    marslib.load()
    X, y, kw = workloads.hinge_search()
    model = mars.fit(X, y, **kw)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(0)
    N = 1_000_000
    Xb = torch.tensor(rng.standard_normal((N, X.shape[1])).astype(np.float32), device=dev)
    Xb = Xb.t().contiguous().t()  # column-major
    Xb.requires_grad_(True)
    beta = torch.tensor(rng.uniform(-1, 1, len(model)).astype(np.float32), device=dev,
                        requires_grad=True)
    knots = torch.tensor(np.nan_to_num(np.asarray(model["hinge"], np.float32)), device=dev,
                         requires_grad=True)

    def step():
        pred = diff.predict(Xb, model, beta, knots)
        pred.sum().backward()

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    line = {"metric": "rows/s (prediction forward + backward, grads in X, beta, knots)",
            "value": N / (ms * 1e-3), "unit": "rows/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (f64 gradient sums)",
            "data": "synthetic", "config": {"workload": WORKLOADS["expand"],
                                            "terms": len(model)}}
    print(json.dumps(line))
    return 0


STAT_KEYS = ("ms_project", "ms_sweep", "ms_dgks", "ms_normalize", "ms_append", "ms_sort",
             "ms_redecide", "ms_gather", "ms_redecide_gpu", "project_flops", "sweep_bytes",
             "evals", "candidates", "redecided", "redecided_flagged", "redecided_degenerate",
             "kernel_launches", "h2d_bytes", "d2h_bytes", "knot_evals", "dgks_fired",
             "evals_exact")


class StopFit(Exception):
    """Raised from the fit's callback to end a profiling run early."""


class EpochSteps:
    """Step boundaries at the epochs of one or more fits.

    Fed by the fit's callback after every epoch (eval + append). The timed
    region opens after `warmup` epochs and closes after `warmup + steps`;
    across it the handle's device span (CUDA events on its stream), the host
    wall time and the counters are accumulated, handle by handle when the
    region spans two fits."""

    def __init__(self, warmup, steps, on_open=None, on_close=None, stop_when_closed=False):
        self.W, self.K = warmup, steps
        self.stop_when_closed = stop_when_closed
        self.on_open, self.on_close = on_open, on_close
        self.done = 0
        self.timing = False
        self.closed = False
        self.algo = None
        self.t_create = []      # (seconds, h2d bytes) of each fit's construction
        self.span_ms = 0.0
        self.wall = 0.0
        self.acc = {k: 0.0 for k in STAT_KEYS}
        self.epoch_ms = []      # device ms of every epoch of the first fit
        self.fit_terms = []     # the current fit's basis size after each of its epochs
        self._prev_span = 0.0
        self.lib = None         # the Counting module of the current fit
        self.walls = None       # (eval, append) host seconds at the region's start

    def _sync(self):
        import torch

        torch.cuda.synchronize()

    def created(self, algo, seconds):
        if self.timing:
            self._fold(self.algo)  # the old handle's share so far
        self.algo = algo
        self.fit_terms = []
        st = algo.stats()
        self.t_create.append((seconds, st["h2d_bytes"]))
        self._prev_span = 0.0
        if self.timing:
            self._base = st  # the new fit's upload ran inside the open region

    def _fold(self, algo):
        st = algo.stats()
        self.span_ms += st["ms_span"] - self._base["ms_span"]
        for k in STAT_KEYS:
            self.acc[k] += st[k] - self._base[k]

    def epoch(self):
        st = self.algo.stats()
        self.epoch_ms.append(st["ms_span"] - self._prev_span)
        self._prev_span = st["ms_span"]
        self.fit_terms.append(self.algo.nbasis())
        self.done += 1
        if not self.timing and not self.closed and self.done == self.W:
            self._sync()
            if self.on_open:
                self.on_open()
            self.timing = True
            self._base = self.algo.stats()
            self._t0 = time.perf_counter()
            if self.lib is not None:
                self.walls = (self.lib.wall_eval, self.lib.wall_append)
        elif self.timing and self.done == self.W + self.K:
            self._sync()
            self.wall += time.perf_counter() - self._t0
            if self.lib is not None and self.walls is not None:
                self.walls = (self.lib.wall_eval - self.walls[0],
                              self.lib.wall_append - self.walls[1])
            self._fold(self.algo)
            self.timing = False
            self.closed = True
            if self.on_close:
                self.on_close()
            if self.stop_when_closed:
                raise StopFit()


def epoch_fit(X, y, kw, precision, steps, shard=False):
    """One fit through the public fit loop with the epoch boundaries of
    `steps`; returns (model, wall seconds, final stats, knot-evals). With
    `shard`, this rank evaluates its block of input columns and the results
    are exchanged (the knot-evals returned and counted are this rank's)."""
    from mars_gb300 import marslib
    from mars_gb300.mars import forward_pass

    def factory(X_, y_, w_, mt):
        t0 = time.perf_counter()
        a = marslib.MarsAlgo(X_, y_, w_, mt)
        a.set_precision(precision)
        steps.created(a, time.perf_counter() - t0)
        return a

    lib = Counting(factory)
    steps.lib = lib
    fit_lib = lib
    if shard:
        from mars_gb300.shard import sharded

        fit_lib = sharded(lib)
    t0 = time.perf_counter()
    try:
        model = forward_pass(fit_lib, X, y, None, callback=lambda *a: steps.epoch(), **kw)
    except StopFit:
        return None, time.perf_counter() - t0, lib.algo.stats(), lib.knot_evals
    wall = time.perf_counter() - t0
    st = lib.algo.stats()
    st["orth_max"], st["rss"] = lib.algo.orth_error()
    st["orth_steps"] = orth_by_step(lib.algo, steps.fit_terms)
    return model, wall, st, lib.knot_evals


def orth_by_step(algo, terms):
    """max |Q^T Q - I| and the RSS (1 - sum(ybo^2), FP64 from Q and y) after
    every epoch of the fit, from the basis sizes `terms` its epochs reached."""
    mx, rss = algo.orth_error_by_terms()
    k = [min(t, len(mx)) - 1 for t in terms if t >= 1]
    return {"terms": [int(j + 1) for j in k],
            "max_abs_QtQ_minus_I": [float(mx[j]) for j in k],
            "rss": [float(rss[j]) for j in k]}


def epoch_grid(X, kw):
    from mars_gb300 import workloads

    n, p = X.shape
    endspan = max(int(n * kw.get("tail_span", 0.02)), 1)
    alpha = 1 / p
    min_span = max(int(-np.log2(-np.log(1 - alpha) / (n * alpha)) / 2.5), 1)
    return endspan, min_span, workloads.knot_evals(n, endspan, min_span)


def parents_of_model(path):
    """Input columns along each basis' parent chain, from a term path."""
    parents = [[]]
    for kind, b, x, _h in path[1:]:
        parents.append(parents[b] + [x])
    return parents


def cpu_epoch_sample(X, y, kw, path, epoch, algo_state, threads, ncols=16, nparents=3):
    """Time the oracle port on a sample of the candidates of `epoch`: the
    basis the fit had built by then (replayed from `path`, the fit's term
    sequence, onto algo_state["algo"] as needed), `ncols` input columns and
    `nparents` allowed parents of each (seeded), one eval call with `threads`
    host threads. Returns (seconds, knot-evals)."""
    import oracle

    if not oracle.available("port"):
        oracle.build(with_reference=False)
    n, p = X.shape
    if algo_state.get("algo") is None:
        w = np.ones(n, dtype=np.float32)
        algo_state["algo"] = oracle.OracleAlgo(X, y, w, kw["max_terms"], kind="port")
        algo_state["epochs"] = 0
        algo_state["row"] = 1
    algo = algo_state["algo"]
    # epochs append one term ('l') or a pair ('+', '-')
    while algo_state["epochs"] < epoch and algo_state["row"] < len(path):
        r = algo_state["row"]
        kind, b, x, h = path[r]
        algo.append(kind, x, b, np.nan if h is None else h)
        r += 1
        if kind == "+" and r < len(path) and path[r][0] == "-":
            kind, b, x, h = path[r]
            algo.append(kind, x, b, h)
            r += 1
        algo_state["row"] = r
        algo_state["epochs"] += 1
    m = algo.nbasis()
    parents = parents_of_model(path[:m])
    max_degree = kw.get("max_degree", 3)
    rng = np.random.default_rng(1000 + epoch)
    mask = np.zeros((p, m), dtype=bool)
    for q in range(ncols):
        i = (epoch * ncols + q) % p
        ok = [j for j in range(m) if len(parents[j]) < max_degree and i not in parents[j]]
        for j in rng.permutation(ok)[:nparents]:
            mask[i, j] = True
    endspan, min_span, grid = epoch_grid(X, kw)
    t0 = time.perf_counter()
    algo.eval(mask, min_span, endspan, False, threads)
    return time.perf_counter() - t0, int(mask.sum()) * grid


def path_epochs(path):
    """Epochs of a fit with this term path: one per linear term or hinge pair."""
    e, r = 0, 1
    while r < len(path):
        r += 2 if path[r][0] == "+" and r + 1 < len(path) and path[r + 1][0] == "-" else 1
        e += 1
    return max(e, 1)


def reference_path(workload_name):
    path = os.path.join(ROOT, "tests", "golden", workload_name + ".json")
    if not os.path.isfile(path):
        return None
    with open(path) as f:
        g = json.load(f)
    return [(r["type"], r["basis"], r["input"], r["hinge"]) for r in g["model"]]


def run_reference_epochs(args):
    """--impl reference on the epoch workload: the oracle port, step k = one
    eval of a sample of epoch W + k's candidates (cpu_epoch_sample)."""
    if RANK != 0:
        return 0
    X, y, kw = workload(args.workload)
    path = reference_path(args.workload)
    base = {"impl": "reference", "metric": METRIC, "config": {"workload": WORKLOADS[args.workload]}}
    if path is None:
        base["unavailable"] = "no reference term path committed for this workload"
        print(json.dumps(base))
        return 0
    threads = cpu_threads()
    state = {}
    epochs = path_epochs(path)
    for e in range(args.warmup):
        cpu_epoch_sample(X, y, kw, path, e % epochs, state, threads)
    total_t, total_k = 0.0, 0
    for k in range(args.steps):
        e = (args.warmup + k) % epochs
        if e < state.get("epochs", 0):
            state.clear()  # past the fit's last epoch: start the basis again
        dt, kn = cpu_epoch_sample(X, y, kw, path, e, state, threads)
        total_t += dt
        total_k += kn
    value = total_k / total_t
    line = dict(base)
    line.update({
        "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "per step: 16 input columns x 3 parents of epoch W+k's "
                                   "candidates on the reference fit's basis at that epoch"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    })
    print(json.dumps(line))
    return 0


def run_epoch_steps(args):
    """Default: the precision-stress fit, one step per epoch (module docstring)."""
    tdist = dist()
    from mars_gb300 import marslib

    marslib.load()
    # bring up torch's CUDA context now: the first torch.cuda.synchronize()
    # costs ~1 s, which would otherwise fall between two of the fit's device
    # events at the opening of the timed region
    import torch

    torch.cuda.init()
    torch.cuda.synchronize()
    X, y, kw = workload(args.workload)
    clocks = Clocks() if RANK == 0 else None
    clk = {}

    def opened():
        if tdist is not None:
            tdist.barrier()
        if clocks:
            clocks.start()

    def closed():
        if clocks:
            clk["v"] = clocks.stop()
        if tdist is not None:
            tdist.barrier()

    steps = EpochSteps(args.warmup, args.steps, opened, closed, args.profile_epochs)
    shard = args.shard and tdist is not None
    fits = []
    while not steps.closed:
        fits.append(epoch_fit(X, y, kw, args.precision, steps, shard))
    if args.profile_epochs:
        acc = steps.acc
        if RANK == 0:
            print(json.dumps({"profile_epochs": [args.warmup, args.warmup + args.steps - 1],
                              "ms_per_step": steps.span_ms / args.steps,
                              "phase_ms_per_step": {k[3:]: acc[k] / args.steps for k in STAT_KEYS
                                                    if k.startswith("ms_")},
                              "host_ms_per_step": {
                                  "eval_call": 1e3 * steps.walls[0] / args.steps,
                                  "append_call": 1e3 * steps.walls[1] / args.steps,
                                  "wall": 1e3 * steps.wall / args.steps},
                              "gpu_launches": int(acc["kernel_launches"]),
                              "per_step": {k: acc[k] / args.steps for k in
                                           ("candidates", "redecided", "redecided_flagged",
                                            "redecided_degenerate", "dgks_fired",
                                            "evals_exact")}}))
        return 0
        if len(fits) > 1 + (args.warmup + args.steps) // 2:
            raise RuntimeError("the fit stops before its epochs reach the timed region")
    clk = clk.get("v")
    model, fit_wall, st, _ = fits[0]
    acc = steps.acc
    t_dev = allmax(tdist, steps.span_ms * 1e-3)
    create_s, create_h2d = steps.t_create[0]
    t_e2e = allmax(tdist, steps.wall + create_s)
    k_all = allsum(tdist, acc["knot_evals"])
    epochs_fit = len(steps.epoch_ms) if len(fits) == 1 else None
    line = {
        "metric": METRIC,
        "value": k_all / t_dev,
        "unit": UNIT,
        "n_gpus": WORLD,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_dev / args.steps,
        "fit_time_s": st["ms_span"] * 1e-3,
        "higher_is_better": True,
        "scaling": "strong" if shard else "weak",
        "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32 with f64 carries; f64 re-decision",
        "precision": args.precision,
        "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload],
                   "step": "one epoch of the fit (eval of every candidate + append); epochs "
                           "%d..%d of the fit timed" % (args.warmup, args.warmup + args.steps - 1),
                   "l2": "not flushed: inputs larger than L2 (X 400 MB)",
                   "parallelism": ("one fit sharded by input column" if shard else "replicas")
                   if WORLD > 1 else "single GPU"},
        "e2e": {"value": k_all / t_e2e, "unit": UNIT,
                "h2d_bytes_per_step": int((acc["h2d_bytes"] + create_h2d) / args.steps),
                "d2h_bytes_per_step": int(acc["d2h_bytes"] / args.steps),
                "note": "host wall time of the timed epochs through the fit loop plus the "
                        "fit's X, y, w upload"},
        "gpu_launches": int(acc["kernel_launches"]),
        "knot_evals_per_step": int(acc["knot_evals"] / args.steps),
        "epochs_in_fit": epochs_fit,
        "terms": len(model),
        "fit_wall_s": fit_wall,
        "roofline": roofline(acc, args.workload, args.precision),
        "phase_ms_per_step": {k[3:]: acc[k] / args.steps for k in STAT_KEYS if
                              k.startswith("ms_")},
        "clocks": clk,
        "orthogonality": {"max_abs_QtQ_minus_I": st["orth_max"], "rss": st["rss"],
                          "per_step": st["orth_steps"]},
    }
    if args.precision == "mixed":
        line["redecided_fraction"] = acc["redecided"] / max(1, acc["candidates"])
    ref = reference_path(args.workload)
    if ref is not None:
        line["term_path_identical_to_reference"] = path_of(model) == ref
    if args.precision == "mixed" and not args.no_compare:
        fsteps = EpochSteps(args.warmup, args.steps)
        fmodel, _, fst, _ = epoch_fit(X, y, kw, "fp64", fsteps, shard)
        fp_timed = sum(fsteps.epoch_ms[args.warmup:args.warmup + args.steps]) * 1e-3
        my_timed = (sum(steps.epoch_ms[args.warmup:args.warmup + args.steps]) * 1e-3
                    if len(fits) == 1 else None)
        line["fp64"] = {"fit_time_s": fst["ms_span"] * 1e-3,
                        "value": (acc["knot_evals"] / fp_timed) if fp_timed else None,
                        "speedup": fst["ms_span"] / max(st["ms_span"], 1e-9),
                        "speedup_timed_epochs": (fp_timed / my_timed) if my_timed else None}
        line["term_path_identical_to_fp64"] = path_of(model) == path_of(fmodel)
        line["orthogonality"]["fp64_max_abs_QtQ_minus_I"] = fst["orth_max"]
        line["orthogonality"]["rss_rel_err_vs_fp64"] = (
            abs(st["rss"] - fst["rss"]) / max(abs(fst["rss"]), 1e-300))
        mine, theirs = st["orth_steps"], fst["orth_steps"]
        line["orthogonality"]["fp64_per_step_max_abs_QtQ_minus_I"] = theirs["max_abs_QtQ_minus_I"]
        line["orthogonality"]["rss_rel_err_vs_fp64_per_step"] = [
            abs(a - b) / max(abs(b), 1e-300) for a, b in zip(mine["rss"], theirs["rss"])]
    if RANK == 0 and not args.no_cpu_baseline:
        threads = cpu_threads()
        e = args.warmup + args.steps // 2
        dt, kn = cpu_epoch_sample(X, y, kw, path_of(model), e, {}, threads)
        line["cpu_baseline"] = {"value": kn / dt, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "16 input columns x 3 parents of epoch %d's "
                                          "candidates, one eval" % e,
                                "seconds": dt}
    if RANK == 0:
        print(json.dumps(line))
    if tdist is not None:
        tdist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.workload in EPOCH_WORKLOADS:
        if args.impl == "reference":
            return run_reference_epochs(args)
        return run_epoch_steps(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "expand":
        return run_expand(args)
    if args.workload == "projection":
        return run_projection(args)
    tdist = dist()
    from mars_gb300 import marslib

    marslib.load()
    X, y, kw = workload(args.workload)
    flush = L2Flush()

    for _ in range(max(args.warmup, 0)):
        flush()
        gpu_fit(X, y, kw, args.precision)

    clocks = Clocks() if RANK == 0 else None
    if tdist is not None:
        tdist.barrier()
    if clocks:
        clocks.start()
    spans, walls, knots, launches, h2d, d2h = [], [], [], [], [], []
    agg = None
    model = None
    for _ in range(args.steps):
        flush()
        model, wall, st, k = gpu_fit(X, y, kw, args.precision)
        spans.append(st["ms_span"] * 1e-3)
        walls.append(wall)
        knots.append(k)
        launches.append(st["kernel_launches"])
        h2d.append(st["h2d_bytes"])
        d2h.append(st["d2h_bytes"])
        if agg is None:
            agg = dict(st)
        else:
            for key in ("ms_project", "ms_sweep", "ms_dgks", "ms_normalize", "ms_append",
                        "ms_sort", "ms_redecide", "ms_gather", "ms_redecide_gpu", "project_flops",
                        "sweep_bytes", "evals", "candidates", "redecided"):
                agg[key] += st[key]
    if tdist is not None:
        tdist.barrier()
    clk = clocks.stop() if clocks else None

    t_dev = allmax(tdist, sum(spans))
    t_wall = allmax(tdist, sum(walls))
    k_all = allsum(tdist, sum(knots))
    line = {
        "metric": METRIC,
        "value": k_all / t_dev,
        "unit": UNIT,
        "n_gpus": WORLD,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_dev / args.steps,
        "fit_time_s": t_dev / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32 with f64 carries; f64 re-decision",
        "precision": args.precision,
        "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "l2": "flushed between steps"
                   if flush.ok else "not flushed (torch unavailable)",
                   "parallelism": "replicas" if WORLD > 1 else "single GPU"},
        "e2e": {"value": k_all / t_wall, "unit": UNIT,
                "h2d_bytes_per_step": int(statistics.mean(h2d)),
                "d2h_bytes_per_step": int(statistics.mean(d2h)),
                "fit_time_s": t_wall / args.steps},
        "gpu_launches": int(sum(launches)),
        "knot_evals_per_step": int(statistics.mean(knots)),
        "terms": len(model),
        "roofline": roofline(agg, args.workload, args.precision),
        "phase_ms_per_step": {k[3:]: agg[k] / args.steps for k in
                              ("ms_project", "ms_dgks", "ms_normalize", "ms_sweep",
                               "ms_append", "ms_sort", "ms_redecide", "ms_gather",
                               "ms_redecide_gpu")},
        "clocks": clk,
        "orthogonality": {"max_abs_QtQ_minus_I": st["orth_max"], "rss": st["rss"]},
    }
    if args.precision == "mixed":
        line["redecided_fraction"] = agg["redecided"] / max(1, agg["candidates"])
    if args.precision == "mixed" and not args.no_compare:
        fp_spans, fp_model = [], None
        for _ in range(max(1, min(args.steps, 2))):
            flush()
            fp_model, _, st, _ = gpu_fit(X, y, kw, "fp64")
            fp_spans.append(st["ms_span"] * 1e-3)
        line["fp64"] = {"fit_time_s": statistics.mean(fp_spans),
                        "value": line["knot_evals_per_step"] / statistics.mean(fp_spans),
                        "speedup": statistics.mean(fp_spans) / (t_dev / args.steps)}
        line["term_path_identical_to_fp64"] = path_of(model) == path_of(fp_model)
        line["orthogonality"]["fp64_max_abs_QtQ_minus_I"] = st["orth_max"]
        line["orthogonality"]["rss_rel_err_vs_fp64"] = (
            abs(line["orthogonality"]["rss"] - st["rss"]) / max(abs(st["rss"]), 1e-300))
    golden = os.path.join(ROOT, "tests", "golden", args.workload + ".json")
    if os.path.isfile(golden):
        with open(golden) as f:
            g = json.load(f)
        want = [(r["type"], r["basis"], r["input"], r["hinge"]) for r in g["model"]]
        line["term_path_identical_to_reference"] = path_of(model) == want
    if RANK == 0 and not args.no_cpu_baseline:
        threads = cpu_threads()
        _, dt, k = cpu_fit(X, y, kw, threads)
        line["cpu_baseline"] = {"value": k / dt, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "one full fit of the same workload",
                                "fit_time_s": dt}
    if RANK == 0:
        print(json.dumps(line))
    if tdist is not None:
        tdist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
