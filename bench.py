"""Throughput of the arc-length path (table build + arc-length sampling) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload uniform_bsplines|ellipses|mixed3d_bsplines|uneven_batch]
                    [--precision plain|mixed|learned]

A step is one pass of the hot path over one batch: createArclengthTable plus
arclengthReverse of every sample of every curve.  Prints ONE JSON line (rank 0).

* ``value``    curves/s with the batch already resident in HBM (device-timed with
               CUDA events around each step on the step's own stream; L2 is
               flushed on that stream before each step, outside the events).
* ``e2e``      the same metric through the public API with host buffers: context
               creation from host arrays (H2D), table, sampling into host memory
               (H2D positions, D2H parameters), destroy; wall clock per step.
               The host arrays are page-locked (filled once, before the loop).
* ``roofline`` for the dominant phase: algorithmic FLOPs (evaluations of the
               plain FP64 method x FLOPs per evaluation as the reference's de
               Boor / ellipse derivative costs them) over the phase's time,
               against the FMA peak of the pipe the form runs on; the library's
               own per-evaluation count beside it.
* ``cpu_baseline`` the reference's CPU algorithm on cost-stratified samples of
               the workload: one thread and all host threads, at the reference's
               default tolerance and at one matched to the accuracy target.
* ``accuracy_vs_fp64_oracle`` every form on a stratified sample of the batch
               plus its hardest curves (most near-duplicate knots, degree 5,
               most intervals, most samples), against the FP64 oracle.
* ``configs``  the other measured workloads (4,096 ellipses and 10,000 uniform
               cubics in plain FP64, 100,000 3D degree-3/5 curves in mixed
               precision), each with its value, roofline, accuracy and CPU baseline.

N > 1 (torchrun): every rank runs its own batch of the full size (weak
scaling, independent curves, no collective on the data path); the step time
is the max over ranks.  ``--impl reference`` times the reference's CPU
implementation of the path on this host (rank 0 only).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "curves/s & samples/s at rel err <=1e-8 vs FP64: learned+mixed vs plain, 1 GB300"

WORKLOADS = {
    # name: (generator kwargs, description)
    "uniform_bsplines": (dict(n=10000, n_ctrl=64, degree=3, dim=2, n_samples=1024),
                         "10,000 clamped uniform cubic 2D B-splines, 64 random-walk control points "
                         "(61 knot intervals), 1,024 samples per curve"),
    "ellipses": (dict(n=4096, n_samples=1000),
                 "4,096 rotated/centred 2D ellipses, a,b~U[0.1,10], 1,000 samples per curve"),
    "mixed3d_bsplines": (dict(n=100_000, n_samples=2048),
                         "100,000 3D clamped B-splines, degree 3|5, 32-256 control points, 2,048 samples"),
    "uneven_batch": (dict(n=1_000_000),
                     "1,000,000 uneven curves (20% ellipses, 80% 2D/3D B-splines degree 2-5, 4-4,096 "
                     "control points, 5% near-duplicate knots), 16-8,192 samples per curve; per-interval "
                     "tolerance 5e-9 for the 1e-8 accuracy target"),
}

# The other workloads, measured beside the headline in the form each is quoted in.
CONFIG_RUNS = (("C1", "ellipses", "plain"), ("C2", "uniform_bsplines", "plain"), ("C3", "mixed3d_bsplines", "mixed"))

# Accuracy bar of each workload (relative length and sample-position error):
# 1e-10 for the FP64 workloads quoted at rtol 1e-10, 1e-8 for the others.
ACCURACY_BAR = {"ellipses": 1e-10, "uniform_bsplines": 1e-10, "mixed3d_bsplines": 1e-8, "uneven_batch": 1e-8}

# The reference's CPU algorithm at its default FP64 tolerance (MAX_ERROR_DOUBLE,
# gcurval/config.h:32) and at an absolute tolerance matched to the 1e-8 target.
REF_MAX_ERROR = 1e-14
MATCHED_MAX_ERROR = 1e-8
# Curves in the CPU baseline's cost-stratified samples: (all host threads, one
# thread) per tolerance, sized for a few seconds each.
CPU_SAMPLES = {
    "uneven_batch": {"default": (512, 48), "matched": (4096, 512)},
    "ellipses": {"default": (4096, 512), "matched": (4096, 512)},
    "uniform_bsplines": {"default": (2048, 256), "matched": (4096, 512)},
    "mixed3d_bsplines": {"default": (1024, 96), "matched": (2048, 192)},
}


# Untimed steps before every timed run: the autotuner's four trial table
# builds of a new batch shape (and form) settle within them.
TUNED_WARMUP = 5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5,
                    help="untimed steps (at least 5: the autotuner's four trial builds settle first)")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="uneven_batch")
    ap.add_argument("--precision", choices=["plain", "mixed", "learned"], default="learned",
                    help="plain FP64, mixed precision, or mixed precision with the learned start depths")
    ap.add_argument("--plain-steps", type=int, default=3,
                    help="timed steps of the plain FP64 form on the same batch, for the speed-up (0: skip)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--config-steps", type=int, default=10, help="timed steps of each per-config run")
    ap.add_argument("--no-configs", action="store_true", help="skip the per-config runs")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the accuracy checks against the oracle")
    ap.add_argument("--no-graph", action="store_true",
                    help="device-resident steps through the ordinary calls instead of the captured CUDA graph")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-curves", type=int, default=0,
                    help="curves of the CPU sample at the default tolerance, all threads (0: the workload's default)")
    ap.add_argument("--n-curves", type=int, default=0, help="override the workload's curve count (profiling runs)")
    ap.add_argument("--split", action="store_true",
                    help="N > 1: split one batch over the ranks by contiguous curve ranges (strong scaling) "
                         "instead of one batch per rank")
    return ap.parse_args()


def make_batch(workload: str, seed: int, n_curves: int = 0):
    from gcurval_gb300 import datasets as ds
    kw, _ = WORKLOADS[workload]
    kw = dict(kw)
    if n_curves:
        kw["n"] = n_curves
    gen = ds.WORKLOADS[workload]
    b = gen(seed=seed, **kw)
    b.sample_positions()
    return b


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- CPU side
def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else platform)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def cpu_sample(batch, n_curves: int):
    """A cost-stratified sample of n_curves curves (largest first), with positions."""
    from gcurval_gb300 import datasets as ds
    sub = batch.subset(ds.stratified_indices(batch, n_curves))
    sub.sample_positions()
    return sub


def run_cpu_reference(sub, nthreads: int, max_error: float = REF_MAX_ERROR):
    """One pass of the reference CPU algorithm over `sub` (table + sampling of
    every sample): (seconds, kind).  The reference's own driver, compiled
    from its tree where that exists, runs at its built-in tolerance: one
    calculator per curve (the driver is instantiated per curve type), taken
    largest first by a pool of nthreads threads.  Other tolerances, and hosts
    without the tree, run the oracle's restatement of it (bit-identical to
    the compiled driver at the same tolerance), whose C thread pool takes
    curves one at a time from a shared counter."""
    from oracle import oracle as orc
    if max_error == REF_MAX_ERROR and orc.reference_available():
        from concurrent.futures import ThreadPoolExecutor
        from gcurval_gb300 import datasets as ds
        order = np.argsort(-ds.cost_proxy(sub), kind="stable")
        items = []
        for i in order:
            p = sub.subset([i])
            p.sample_positions()
            items.append((p, orc.Reference(p, nthreads=1)))
        run = lambda it: it[1].run(it[0].n_samples, it[0].positions, True, 0)
        t0 = time.perf_counter()
        if nthreads <= 1:
            for it in items:
                run(it)
        else:
            with ThreadPoolExecutor(max_workers=nthreads) as ex:
                list(ex.map(run, items))  # ctypes releases the GIL during each call
        return time.perf_counter() - t0, "reference"
    t0 = time.perf_counter()
    o = orc.Oracle(sub, max_error=max_error, nthreads=nthreads)
    o.reverse(sub.n_samples, sub.positions, True, 0)
    return time.perf_counter() - t0, "port"


def cpu_baseline(batch, workload: str, nthreads: int, n_default: int = 0) -> dict:
    """The reference's CPU algorithm on cost-stratified samples of the batch:
    all host threads and one thread, at the default and at the matched
    tolerance.  ``value`` is all threads at the default tolerance.
    n_default overrides that run's sample size (and scales the others)."""
    sizes = CPU_SAMPLES[workload]
    scale = n_default / sizes["default"][0] if n_default else 1.0
    runs = []
    for tol_name, max_error in (("default", REF_MAX_ERROR), ("matched", MATCHED_MAX_ERROR)):
        n_all, n_one = (max(1, int(round(x * scale))) for x in sizes[tol_name])
        for threads, n in ((nthreads, n_all), (1, n_one)):
            sub = cpu_sample(batch, n)
            secs, kind = run_cpu_reference(sub, threads, max_error)
            nseg = int(sub.n_segments.sum())
            runs.append({"threads": threads, "tolerance": tol_name, "max_error": max_error, "kind": kind,
                         "curves": int(sub.n_curve), "samples": int(sub.total_samples), "intervals": nseg,
                         "seconds": round(secs, 3), "curves_per_s": round(sub.n_curve / secs, 3),
                         "samples_per_s": round(sub.total_samples / secs, 1),
                         "intervals_per_s": round(nseg / secs, 1)})
    head = runs[0]
    return {"value": head["curves_per_s"], "unit": "curves/s", "cores": nthreads, "kind": head["kind"],
            "sample": (f"{head['curves']} curves, a cost-stratified sample of the workload ({head['samples']} "
                       f"samples, {head['intervals']} knot intervals), table + sampling, all {nthreads} host "
                       f"threads, absolute tolerance {REF_MAX_ERROR:g} (the reference's default)"),
            "samples_per_s": head["samples_per_s"], "intervals_per_s": head["intervals_per_s"],
            "cpu_model": cpu_model(), "nproc": os.cpu_count(), "runs": runs}


def accuracy_vs_oracle(sub, forms: dict, rtol: float, bar: float, model=None) -> dict:
    """Relative total-length error and sample-position error |s(u) - target| / L
    of the library's forms on `sub` against the FP64 oracle (the reference's
    CPU algorithm restated, its tolerance scaled to each curve's size),
    maxima over the subset.  forms: name -> (precision, learned)."""
    import gcurval_gb300 as g
    from oracle import oracle as orc
    t0 = time.perf_counter()
    o = orc.ScaledOracle(sub)
    Lo = o.lengths()
    tgt = sub.positions * np.repeat(Lo, sub.n_samples)
    Lrep = np.maximum(np.repeat(Lo, sub.n_samples), 1e-300)
    out = {}
    for name, (prec, learned) in forms.items():
        calc = g.ArclengthCalculateGpu.from_batch(sub, precision=prec, rtol=rtol, learned=learned)
        if learned:
            calc.set_learned_model(model)
        try:
            calc.createArclengthTable()
            L = calc.getAllCurveArclengths()
            u = calc.arclengthReverse(sub.n_samples, sub.positions, True, g.GCV_HOST).us
        finally:
            calc.close()
        s = o.s_at(sub.n_samples, u)
        le = np.abs(L - Lo) / np.maximum(Lo, 1e-300)
        se = np.abs(s - tgt) / Lrep if s.size else np.zeros(1)
        out[name] = {"max_rel_length_err": float(np.max(le)), "max_rel_sample_err": float(np.max(se)),
                     "worst_curve_samples": int(np.argmax(se)) if s.size else -1,
                     "bar": bar, "within_bar": bool(np.max(le) <= bar and np.max(se) <= bar)}
    return {"curves": int(sub.n_curve), "samples": int(sub.total_samples),
            "intervals": int(sub.n_segments.sum()), "forms": out, "seconds": round(time.perf_counter() - t0, 2),
            "oracle": "oracle/ C restatement of ArclengthCalculateCpu, FP64, MAX_ERROR 1e-16 x control-polygon length"}


def accuracy_subset(batch, n_stratified: int, k_hard: int):
    from gcurval_gb300 import datasets as ds
    sub = batch.subset(ds.accuracy_subset_indices(batch, n_stratified, k_hard))
    sub.sample_positions()
    return sub


# --------------------------------------------------------- FLOP counting
def flops_per_eval(batch) -> float:
    """This library's FP64-equivalent FLOPs of one |C'| evaluation (add, mul,
    sqrt 1, FMA 2) on its per-interval polynomials, batch mean over curves."""
    p = batch.degree.astype(np.float64)
    d = batch.dim.astype(np.float64)
    bs = d * 2.0 * np.maximum(p - 1, 0) + (2.0 * d - 1.0) + 1.0  # Horner, squared norm, sqrt
    ell = 1.0 + 2.0 + 2.0 + 1.0 + 20.0  # s^2, fma, sqrt, scale + sinpi (counted as 20)
    return float(np.mean(np.where(batch.kind == 0, ell, bs)))


def survey_flops_per_eval(batch, weight) -> float:
    """FLOPs of one |C'(t)| evaluation as the reference computes it (de Boor
    basis and derivative, samples/sample2_bspline/BSpline.h:50-96 with
    gcurval/base/functors.inl.h:51-63; ellipse 12): B-spline of degree p in
    dimension D: 2(p-1) + 2.5 p(p-1) + 2 + 4p + D(2p+1) + 2D + 4 (51 for a
    2D cubic, 101 for a 3D quintic).  Mean over curves weighted by `weight`
    (intervals for the length phase, samples for sampling)."""
    p = batch.degree.astype(np.float64)
    d = batch.dim.astype(np.float64)
    bs = 2 * (p - 1) + 2.5 * p * (p - 1) + 2 + 4 * p + d * (2 * p + 1) + 2 * d + 4
    f = np.where(batch.kind == 0, 12.0, bs)
    w = np.asarray(weight, np.float64)
    return float(np.sum(f * w) / max(np.sum(w), 1.0))


# ------------------------------------------------------- multi-rank glue
def max_over_ranks(x: float, dist, device) -> float:
    """The maximum of x over the ranks (x itself without a process group)."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: int, ms_per_step_max: float, world: int) -> float:
    """Whole-job units/s: every rank processes its own batch of units_per_rank
    (weak scaling), a step lasts as long as the slowest rank."""
    return world * units_per_rank / (ms_per_step_max * 1e-3)


# --------------------------------------------------------------- our arm
class Resident:
    """A batch, its sample counts and positions and an output array, in HBM."""

    def __init__(self, batch, dev):
        import torch
        tk = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
        self.batch = batch
        self.arr = (tk(batch.kind, torch.uint8), tk(batch.degree, torch.uint8), tk(batch.dim, torch.uint8),
                    tk(batch.knot_off, torch.int64), tk(batch.knots, torch.float64),
                    tk(batch.ctrl_off, torch.int64), tk(batch.ctrl, torch.float64))
        self.cnt = tk(batch.n_samples, torch.int32)
        self.pos = tk(batch.positions, torch.float64)
        self.out = torch.empty(batch.total_samples, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()


class Bench:
    """Device-resident timing of one batch: every call of the library, the
    L2 flush and the CUDA events run on one stream of this object's own, so
    the flush is ordered before each step and the events bracket it."""

    def __init__(self, dev, local, dist, use_graph=True):
        import torch
        self.torch = torch
        self.dev = dev
        self.local = local
        self.dist = dist
        self.use_graph = use_graph
        self.stream = torch.cuda.Stream(device=dev)
        with torch.cuda.stream(self.stream):
            self.flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def run(self, res, prec, steps, warmup, learned_on=False, model=None, clocks=False, mapping="lane"):
        """Times `steps` table builds + samplings (after `warmup` untimed ones)."""
        import gcurval_gb300 as g
        torch = self.torch
        b = res.batch
        with torch.cuda.stream(self.stream):
            calc = g.ArclengthCalculateGpu.from_device_batch(*res.arr, precision=prec, rtol=b.rtol,
                                                             collect_stats=True, learned=learned_on,
                                                             stream=self.stream, mapping=mapping)
            if learned_on:
                calc.set_learned_model(model)

            def step():
                if self.use_graph:
                    calc.stepGraph(res.cnt, res.pos, res.out, True, g.GCV_RETURN_US)
                else:
                    calc.createArclengthTable()
                    calc.arclengthReverseInto(res.cnt, res.pos, res.out, True, g.GCV_RETURN_US)

            for _ in range(warmup):
                step()
            self.stream.synchronize()
            launches0 = calc.stats()["n_launches"]
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
            r = {"ms_len": [], "ms_samp": [], "ms_setup": [], "n_newton": [], "n_panels": [], "ms_learned": []}
            if self.dist:
                self.dist.barrier()
            torch.cuda.synchronize()
            with ClockSampler(self.local) as clk:
                for i in range(steps):
                    self.flush.zero_()
                    evs[i][0].record(self.stream)
                    step()
                    evs[i][1].record(self.stream)
                    st = calc.stats()  # synchronises; outside the events
                    r["ms_len"].append(st["ms_length"])
                    r["ms_samp"].append(st["ms_sample"])
                    r["ms_setup"].append(st["ms_setup"] + st["ms_scan"])
                    r["n_newton"].append(st["n_newton"])
                    r["n_panels"].append(st["n_panels"])
                    r["ms_learned"].append(st["ms_learned"])
                self.stream.synchronize()
            if self.dist:
                self.dist.barrier()
            total_ms = max_over_ranks(float(sum(x.elapsed_time(y) for x, y in evs)), self.dist, self.dev)
            st1 = calc.stats()
            r["launches"] = st1["n_launches"] - launches0
            r["leaves"] = st1["n_leaves"]
            r["deep"] = st1["n_deep_segments"]
            r["capped"] = st1["n_capped"]
            slots = ["ellipse"] + [f"p{p}d{d}" for d in (2, 3) for p in range(1, 6)]
            r["launch_shapes"] = {"tuned": bool(st1["tuned"]),
                                  "length_workers_per_sm": {n: v for n, v in zip(slots, st1["length_blocks_per_sm_code"])},
                                  "deep_workers_per_sm": st1["length_blocks_per_sm"],
                                  "sample_threads": st1["sample_threads"],
                                  "sample_blocks_per_sm": st1["sample_blocks_per_sm"]}
            r["ms_per_step"] = total_ms / steps
            r["steps"] = steps
            r["clocks"] = clk.summary() if clocks else None
            calc.close()
        return r


def roofline_of(batch, r, plain_r, is_plain: bool, workload: str, precision: str, fp64_peak: float,
                fp32_peak: float, hbm_peak):
    """Roofline of the dominant phase of run r (the larger of length walk and
    sampling).  achieved = the plain FP64 method's integrand evaluations for
    the batch (plain_r's panels x 16 and Newton iterations x 10) x the
    reference's FLOPs per evaluation, over the phase's time; the library's
    own count (its own evaluations x its cheaper per-evaluation FLOPs) is
    given beside it."""
    n_samples = batch.total_samples
    fpe = flops_per_eval(batch)
    ms_inf = r["ms_learned"]
    ms_l = float(np.mean([a - b for a, b in zip(r["ms_len"], ms_inf)]))
    ms_s = float(np.mean(r["ms_samp"]))
    newton, panels = float(np.mean(r["n_newton"])), float(np.mean(r["n_panels"]))
    # a Newton iteration: 8 Gauss nodes, the speed and slope at v and at the Newton point
    own_samp = newton * (8 * (fpe + 4.0) + 2 * (fpe + 4.0)) + n_samples * 20.0
    own_len = panels * (16 * (fpe + 2.0) + 40.0)
    src = plain_r if plain_r is not None else r
    f_len = survey_flops_per_eval(batch, batch.n_segments)
    f_smp = survey_flops_per_eval(batch, batch.n_samples)
    sv_len = float(np.mean(src["n_panels"])) * 16.0 * f_len
    sv_samp = float(np.mean(src["n_newton"])) * 10.0 * f_smp
    if ms_s >= ms_l:
        dom, flops, own, ms = "k_sample", sv_samp, own_samp, ms_s
        bytes_alg = n_samples * (8 + 8 + 8) + batch.n_curve * 8
        units = n_samples
    else:
        dom, flops, own, ms = "k_length", sv_len, own_len, ms_l
        bytes_alg = batch.knots.nbytes + batch.ctrl.nbytes + int(batch.n_segments.sum()) * 8
        units = float(batch.n_segments.sum())
    peak = fp64_peak if is_plain else fp32_peak
    achieved = flops / (ms * 1e-3) / 1e12
    traffic = None
    prof = os.path.join(ROOT, "profiles", "traffic_per_unit.json")
    if os.path.exists(prof):
        try:
            tpu = json.load(open(prof)).get(f"{dom}:{workload}:{precision}")
            if tpu:
                traffic = float(tpu) * units
        except (ValueError, OSError):
            traffic = None
    return {
        "kernel": dom, "bound": "fp64" if is_plain else "fp32",
        "achieved": round(achieved, 4), "peak": round(peak, 4), "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
        "peak_source": "measured in-run by gcv_measure_fma_peak (FMA probe kernel)",
        "work": ("evaluations of the plain FP64 method (panels x 16 + Newton iterations x 10) x FLOPs per "
                 "evaluation of the reference's de Boor / ellipse derivative"),
        "flops_per_eval_reference": round(f_smp if dom == "k_sample" else f_len, 3),
        "traffic": traffic, "ms_per_launch": round(ms, 4), "algorithmic_flops_per_launch": flops,
        "own_count": {"flops_per_eval": round(fpe, 3), "flops": own, "achieved": round(own / (ms * 1e-3) / 1e12, 4),
                      "frac": round(own / (ms * 1e-3) / 1e12 / peak, 4),
                      "work": "this form's own panels / Newton iterations x its FLOPs per evaluation"},
        "hbm": {"achieved_gbs": round(bytes_alg / (ms * 1e-3) / 1e9, 2), "peak_gbs": hbm_peak,
                "frac": round(bytes_alg / (ms * 1e-3) / 1e9 / hbm_peak, 4) if hbm_peak else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "phases_ms": {"length": round(ms_l, 4), "sample": round(ms_s, 4),
                      "setup_scan": round(float(np.mean(r["ms_setup"])), 4),
                      "network_inference": round(float(np.mean(ms_inf)), 4)},
        "work_per_step": {"panels": panels, "newton_iterations": newton, "leaves": int(r["leaves"]),
                          "segments": int(batch.n_segments.sum()), "capped_panels": int(r["capped"]),
                          "plain_panels": float(np.mean(src["n_panels"])),
                          "plain_newton_iterations": float(np.mean(src["n_newton"]))},
        "fp64_peak_tflops": round(fp64_peak, 3), "fp32_peak_tflops": round(fp32_peak, 2),
    }


def hbm_peak_gbs():
    mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(mp):
        try:
            return json.load(open(mp)).get("hbm_gbs")
        except (ValueError, OSError):
            return None
    return None


def measure_config(name, workload, precision, bench, args, fp64_peak, fp32_peak, nthreads):
    """Value, roofline, accuracy and CPU baseline of one other workload."""
    import gcurval_gb300 as g
    batch = make_batch(workload, seed=0)
    res = Resident(batch, bench.dev)
    prec = g.GCV_PLAIN_FP64 if precision == "plain" else g.GCV_MIXED
    r = bench.run(res, prec, args.config_steps, TUNED_WARMUP)
    plain_r = None if precision == "plain" else bench.run(res, g.GCV_PLAIN_FP64, 2, TUNED_WARMUP)
    del res
    value = batch.n_curve / (r["ms_per_step"] * 1e-3)
    out = {"workload": f"{workload}: {WORKLOADS[workload][1]}", "precision": precision, "rtol": batch.rtol,
           "value": round(value, 3), "unit": "curves/s", "ms_per_step": round(r["ms_per_step"], 4),
           "steps": r["steps"], "warmup": TUNED_WARMUP,
           "samples_per_s": round(batch.total_samples / (r["ms_per_step"] * 1e-3), 1),
           "roofline": roofline_of(batch, r, plain_r, precision == "plain", workload, precision, fp64_peak,
                                   fp32_peak, hbm_peak_gbs())}
    if plain_r is not None:
        out["plain_fp64_same_batch"] = {"value": round(batch.n_curve / (plain_r["ms_per_step"] * 1e-3), 3),
                                        "ms_per_step": round(plain_r["ms_per_step"], 4)}
    if not args.no_accuracy:
        sub = accuracy_subset(batch, 400, 40)
        out["accuracy_vs_fp64_oracle"] = accuracy_vs_oracle(sub, {precision: (prec, False)}, batch.rtol,
                                                            ACCURACY_BAR[workload])
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(batch, workload, nthreads)
    return out


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args)
        if dist:
            dist.destroy_process_group()
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import gcurval_gb300 as g
    from gcurval_gb300 import _lib

    precision = g.GCV_PLAIN_FP64 if args.precision == "plain" else g.GCV_MIXED
    use_learned = args.precision == "learned"
    model = None
    if use_learned:
        from gcurval_gb300 import learned as _learned
        model = _learned.load_model()
    split = args.split and world > 1
    if split:
        # one batch, this rank's contiguous share of its curves
        from gcurval_gb300 import sharding
        full = make_batch(args.workload, seed=0, n_curves=args.n_curves)
        _, _, batch = sharding.shard(full, rank, world)
        job_curves, job_samples = full.n_curve, full.total_samples
        del full
    else:
        batch = make_batch(args.workload, seed=rank, n_curves=args.n_curves)
        job_curves, job_samples = world * batch.n_curve, world * batch.total_samples
    pos = batch.positions
    n_curves, n_samples = batch.n_curve, batch.total_samples
    rtol = batch.rtol
    nthreads = os.cpu_count() or 1

    # ---- device-resident arm ------------------------------------------------
    bench = Bench(dev, local, dist, use_graph=not args.no_graph)
    res = Resident(batch, dev)
    main_r = bench.run(res, precision, args.steps, max(args.warmup, 5), learned_on=use_learned, model=model,
                       clocks=True)
    plain_r = mixed_r = hw_r = None
    if precision != g.GCV_PLAIN_FP64 and args.plain_steps > 0:
        plain_r = bench.run(res, g.GCV_PLAIN_FP64, args.plain_steps, TUNED_WARMUP)
        if use_learned:
            # the same mixed-precision walk without the network: what the network gains
            mixed_r = bench.run(res, g.GCV_MIXED, args.plain_steps, TUNED_WARMUP)
        if precision == g.GCV_MIXED:
            # the length walk's other mapping: one half-warp per knot interval
            hw_r = bench.run(res, precision, args.plain_steps, TUNED_WARMUP, learned_on=use_learned, model=model,
                             mapping="half_warp")
    del res
    ms_per_step = main_r["ms_per_step"]
    value = job_curves / (ms_per_step * 1e-3)
    samples_per_s = job_samples / (ms_per_step * 1e-3)
    fp64_peak = _lib.measure_fma_peak(0)
    fp32_peak = _lib.measure_fma_peak(1)
    roofline = roofline_of(batch, main_r, plain_r if precision != g.GCV_PLAIN_FP64 else None,
                           precision == g.GCV_PLAIN_FP64, args.workload, args.precision, fp64_peak, fp32_peak,
                           hbm_peak_gbs())

    # ---- end-to-end through the public API with host buffers -----------------
    # The step's inputs (curve arrays, sample counts and positions) and its
    # output live in page-locked host memory, filled once before the loop.
    e2e_t, parts = [], []
    hb = dataclasses.replace(batch, **{f: g.pinned_copy(getattr(batch, f)) for f in
                                       ("kind", "degree", "dim", "knot_off", "knots", "ctrl_off", "ctrl", "n_samples")})
    h_pos = g.pinned_copy(pos)
    h_out = g.pinned_empty(n_samples, np.float64)
    def e2e_steps(in_place):
        times, split = [], []
        for i in range(max(args.e2e_steps, 1) + 1):
            if dist:
                dist.barrier()
            t = [time.perf_counter()]
            c2 = g.ArclengthCalculateGpu.from_batch(hb, precision=precision, rtol=batch.rtol, learned=use_learned,
                                                    host_in_place=in_place)
            if use_learned:
                c2.set_learned_model(model)
            t.append(time.perf_counter())
            c2.createArclengthTable()
            t.append(time.perf_counter())
            c2.arclengthReverseInto(hb.n_samples, h_pos, h_out, True, g.GCV_RETURN_US)
            t.append(time.perf_counter())
            c2.close()
            t.append(time.perf_counter())
            if i > 0:
                times.append(t[-1] - t[0])
                split.append(np.diff(t) * 1e3)
        return (max_over_ranks(float(np.mean(times)), dist, dev),
                dict(zip(["create", "table", "sample", "destroy"], np.round(np.mean(split, axis=0), 3).tolist())))

    # curve arrays read in place by the table build (host_in_place), and
    # copied to the device at creation
    e2e_s, e2e_parts = e2e_steps(True)
    e2e_copy_s, e2e_copy_parts = e2e_steps(False)
    h2d = batch.nbytes() + batch.n_samples.nbytes + pos.nbytes
    d2h = h_out.nbytes
    del hb, h_pos, h_out

    # ---- accuracy, CPU baseline and the other configs (rank 0, N = 1 only) ---
    cpu = acc = None
    configs = None
    if rank == 0 and world == 1:
        if not args.no_accuracy:
            sub = accuracy_subset(batch, 1000, 250)
            forms = {args.precision: (precision, use_learned)}
            if use_learned:
                forms["mixed"] = (g.GCV_MIXED, False)
            if precision != g.GCV_PLAIN_FP64:
                forms["plain"] = (g.GCV_PLAIN_FP64, False)
            acc = accuracy_vs_oracle(sub, forms, batch.rtol, ACCURACY_BAR[args.workload], model)
            acc["subset"] = ("1,000 curves cost-stratified over the batch plus its hardest: the 250 with the most "
                             "near-duplicate knots, the 250 degree-5 curves with the most, the 250 with the most "
                             "knot intervals, the 250 with the most samples, 25 random curves of every code")
        if not args.no_cpu_baseline:
            cpu = cpu_baseline(batch, args.workload, nthreads, args.cpu_sample_curves)
        if not args.no_configs and args.workload == "uneven_batch" and not args.n_curves:
            del batch
            _lib.release_cached_memory()
            torch.cuda.empty_cache()
            configs = {}
            for name, wl, pr in CONFIG_RUNS:
                configs[name] = measure_config(name, wl, pr, bench, args, fp64_peak, fp32_peak, nthreads)
                _lib.release_cached_memory()
                torch.cuda.empty_cache()
    plain = None
    if plain_r is not None:
        pv = job_curves / (plain_r["ms_per_step"] * 1e-3)
        plain = {"value": round(pv, 3), "unit": "curves/s", "ms_per_step": round(plain_r["ms_per_step"], 4),
                 "steps": args.plain_steps, "warmup": TUNED_WARMUP, "rtol": rtol,
                 "samples_per_s": round(job_samples / (plain_r["ms_per_step"] * 1e-3), 1),
                 "phases_ms": {"length": round(float(np.mean(plain_r["ms_len"])), 4),
                               "sample": round(float(np.mean(plain_r["ms_samp"])), 4),
                               "setup_scan": round(float(np.mean(plain_r["ms_setup"])), 4)},
                 "speedup_of_this_form": round(value / pv, 3)}
    gain = None
    if mixed_r is not None:
        mv = job_curves / (mixed_r["ms_per_step"] * 1e-3)
        ms_inf = main_r["ms_learned"]
        gain = {"mixed_without_network": {"value": round(mv, 3), "unit": "curves/s",
                                          "ms_per_step": round(mixed_r["ms_per_step"], 4),
                                          "panels": float(np.mean(mixed_r["n_panels"])),
                                          "length_ms": round(float(np.mean(mixed_r["ms_len"])), 4)},
                "with_network": {"panels": float(np.mean(main_r["n_panels"])),
                                 "length_ms": round(float(np.mean([a - b for a, b in zip(main_r["ms_len"], ms_inf)])), 4),
                                 "inference_ms": round(float(np.mean(ms_inf)), 4)},
                "panels_saved_frac": round(1.0 - float(np.mean(main_r["n_panels"])) / float(np.mean(mixed_r["n_panels"])), 4),
                "speedup_over_mixed": round(value / mv, 4)}

    mapping_cmp = None
    if hw_r is not None:
        ms_l_lane = float(np.mean([a - b for a, b in zip(main_r["ms_len"], main_r["ms_learned"])]))
        ms_l_hw = float(np.mean([a - b for a, b in zip(hw_r["ms_len"], hw_r["ms_learned"])]))
        mapping_cmp = {"lane_per_interval": {"length_ms": round(ms_l_lane, 4), "ms_per_step": round(ms_per_step, 4)},
                       "half_warp_per_interval": {"length_ms": round(ms_l_hw, 4),
                                                  "ms_per_step": round(hw_r["ms_per_step"], 4)},
                       "length_speedup_of_lane": round(ms_l_hw / ms_l_lane, 4)}
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "curves/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 5), "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
            "scaling": "strong" if split else "weak", "vs_baseline": None,
            "dtype": "f64" if precision == g.GCV_PLAIN_FP64 else ("f32+f64+bf16" if use_learned else "f32+f64"),
            "data": "synthetic: seeded generator (numpy default_rng, seed = rank)",
            "config": {"workload": f"{args.workload}: {WORKLOADS[args.workload][1]}",
                       "precision": args.precision, "rtol": rtol,
                       "curves_per_gpu": n_curves, "samples_per_gpu": n_samples,
                       "l2": "flushed between timed steps (256 MB write on the step's stream, untimed)",
                       "step": "one captured CUDA graph per step (gcv_step_graph)" if not args.no_graph else
                               "createArclengthTable + arclengthReverseInto",
                       "parallelism": (f"split x{world}: contiguous curve ranges of one batch, balanced by cost "
                                       "(no collective on the data path)") if split else
                                      f"replicas x{world} (independent curves, no collective)"},
            "samples_per_s": round(samples_per_s, 1),
            "e2e": {"value": round(job_curves / e2e_s, 3), "unit": "curves/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "samples_per_s": round(job_samples / e2e_s, 1),
                    "ms_per_step": round(e2e_s * 1e3, 3), "breakdown_ms": e2e_parts,
                    "inputs": "page-locked host arrays: curve data read in place by the table build "
                              "(host_in_place), positions and parameters by the sampling kernels",
                    "copying_create": {"value": round(job_curves / e2e_copy_s, 3),
                                       "ms_per_step": round(e2e_copy_s * 1e3, 3),
                                       "breakdown_ms": e2e_copy_parts}},
            "gpu_launches": int(main_r["launches"]),
            "launch_shapes": main_r["launch_shapes"],
            "roofline": roofline,
            "cpu_baseline": cpu,
            "accuracy_vs_fp64_oracle": acc,
            "plain_fp64_same_batch": plain,
            "learned_gain": gain,
            "length_walk_mapping": mapping_cmp,
            "configs": configs,
            "clocks": main_r["clocks"],
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def reference_arm(args):
    """The reference's CPU implementation of the path on this host's cores:
    each step one pass (table + sampling) over the same cost-stratified
    sample the cpu_baseline leg times, all host threads, the reference's
    default tolerance."""
    nthreads = os.cpu_count() or 1
    batch = make_batch(args.workload, seed=0, n_curves=args.n_curves)
    sub = cpu_sample(batch, args.cpu_sample_curves or CPU_SAMPLES[args.workload]["default"][0])
    times, kind = [], None
    for i in range(max(args.warmup, 3) + args.steps):
        secs, kind = run_cpu_reference(sub, nthreads, REF_MAX_ERROR)
        if i >= max(args.warmup, 3):
            times.append(secs)
    per = float(np.mean(times))
    value = sub.n_curve / per
    nseg = int(sub.n_segments.sum())
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "curves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(per * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded generator (numpy default_rng, seed 0)",
        "config": {"workload": f"{args.workload}: {WORKLOADS[args.workload][1]}", "precision": "plain",
                   "sample_curves": sub.n_curve, "max_error": REF_MAX_ERROR},
        "samples_per_s": round(sub.total_samples / per, 1),
        "intervals_per_s": round(nseg / per, 1),
        "cpu_baseline": {"value": round(value, 3), "unit": "curves/s", "cores": nthreads, "kind": kind,
                         "sample": f"{sub.n_curve} curves, a cost-stratified sample of the workload "
                                   f"({sub.total_samples} samples, {nseg} knot intervals) per step, table + "
                                   f"sampling, all host threads, absolute tolerance {REF_MAX_ERROR:g}",
                         "cpu_model": cpu_model(), "nproc": os.cpu_count()},
        "e2e": {"value": round(value, 3), "unit": "curves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
