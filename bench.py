"""Throughput of the arc-length path (table build + arc-length sampling) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload uniform_bsplines|ellipses|mixed3d_bsplines|uneven_batch]
                    [--precision plain|mixed]

A step is one pass of the hot path over one batch: createArclengthTable plus
arclengthReverse of every sample of every curve.  Prints ONE JSON line (rank 0).

* ``value``  curves/s with the batch already resident in HBM (device-timed with
             CUDA events around each step; L2 is flushed between steps).
* ``e2e``    the same metric through the public API with host buffers: context
             creation from host arrays (H2D), table, sampling into host memory
             (H2D positions, D2H parameters), destroy; wall clock per step.
* ``roofline`` for the dominant kernel, ``cpu_baseline`` (the reference's CPU
             algorithm on a bounded sample, all host threads), ``clocks``.

N > 1 (torchrun): every rank runs its own batch of the full size (weak
scaling, independent curves, no collective on the data path); the step time
is the max over ranks.  ``--impl reference`` times the reference's CPU
implementation of the path on this host (rank 0 only).
"""
from __future__ import annotations

import argparse
import json
import os
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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="uneven_batch")
    ap.add_argument("--precision", choices=["plain", "mixed", "learned"], default="learned",
                    help="plain FP64, mixed precision, or mixed precision with the learned start depths")
    ap.add_argument("--plain-steps", type=int, default=3,
                    help="timed steps of the plain FP64 form on the same batch, for the speed-up (0: skip)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-graph", action="store_true",
                    help="device-resident steps through the ordinary calls instead of the captured CUDA graph")
    ap.add_argument("--cpu-sample-curves", type=int, default=0, help="curves in the CPU-baseline sample (0: auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n-curves", type=int, default=0, help="override the workload's curve count (profiling runs)")
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
def cpu_sample(batch, n_curves: int):
    idx = np.linspace(0, batch.n_curve - 1, n_curves).astype(np.int64)
    sub = batch.subset(np.unique(idx))
    sub.sample_positions()
    return sub


def _groups(batch):
    """Curve subsets of one (kind, degree, dim): the reference's CPU driver
    is instantiated per curve type, as its sample programs are."""
    key = batch.kind.astype(np.int64) * 100 + batch.degree.astype(np.int64) * 10 + batch.dim.astype(np.int64)
    return [batch.subset(np.nonzero(key == k)[0]) for k in np.unique(key)]


def run_cpu_reference(sub, nthreads: int, prefer_reference: bool = True):
    """One pass of the reference CPU algorithm over `sub` (table + sampling of
    every sample): (seconds, kind).  Batches that mix curve types run one
    reference calculator per type, back to back."""
    from oracle import oracle as orc
    if prefer_reference and orc.reference_available():
        parts = _groups(sub)
        for p in parts:
            p.sample_positions()
        refs = [orc.Reference(p, nthreads=nthreads) for p in parts]
        t0 = time.perf_counter()
        for p, ref in zip(parts, refs):
            ref.run(p.n_samples, p.positions, True, 0)
        return time.perf_counter() - t0, "reference"
    t0 = time.perf_counter()
    o = orc.Oracle(sub, nthreads=nthreads)
    o.reverse(sub.n_samples, sub.positions, True, 0)
    return time.perf_counter() - t0, "port"


def accuracy_vs_oracle(sub, precision, rtol, model=None):
    """Relative total-length error and sample-position error |s(u) - target| / L
    of the library on `sub` against the FP64 oracle (the reference's CPU
    algorithm restated), maxima over the subset."""
    import gcurval_gb300 as g
    from oracle import oracle as orc
    calc = g.ArclengthCalculateGpu.from_batch(sub, precision=precision, rtol=rtol, learned=model is not None)
    if model is not None:
        calc.set_learned_model(model)
    try:
        calc.createArclengthTable()
        L = calc.getAllCurveArclengths()
        u = calc.arclengthReverse(sub.n_samples, sub.positions, True, g.GCV_HOST).us
    finally:
        calc.close()
    o = orc.Oracle(sub)
    Lo = o.lengths()
    s = o.s_at(sub.n_samples, u)
    tgt = sub.positions * np.repeat(Lo, sub.n_samples)
    Lrep = np.maximum(np.repeat(Lo, sub.n_samples), 1e-300)
    return {"curves": int(sub.n_curve), "samples": int(sub.total_samples),
            "max_rel_length_err": float(np.max(np.abs(L - Lo) / np.maximum(Lo, 1e-300))),
            "max_rel_sample_err": float(np.max(np.abs(s - tgt) / Lrep)) if s.size else 0.0,
            "oracle": "oracle/ C restatement of ArclengthCalculateCpu, FP64"}


def auto_cpu_curves(batch, nthreads: int, target_s: float) -> int:
    """Curves of the CPU sample: a pilot of 32 curves spread over the batch,
    timed, scaled to about `target_s` seconds on `nthreads` threads."""
    pilot = cpu_sample(batch, min(32, batch.n_curve))
    secs, _ = run_cpu_reference(pilot, nthreads)
    n = int(pilot.n_curve * target_s / max(secs, 1e-3))
    return int(max(16, min(batch.n_curve, n)))


# --------------------------------------------------------------- our arm
def flops_per_eval(batch) -> float:
    """FP64 flops of one |C'| evaluation (add/mul/sqrt/div 1, FMA 2), batch mean."""
    p = batch.degree.astype(np.float64)
    d = batch.dim.astype(np.float64)
    bs = d * 2.0 * np.maximum(p - 1, 0) + (2.0 * d - 1.0) + 1.0  # Horner, squared norm, sqrt
    ell = 1.0 + 2.0 + 2.0 + 1.0 + 20.0  # s^2, fma, sqrt, scale + sinpi (counted as 20)
    return float(np.mean(np.where(batch.kind == 0, ell, bs)))


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
    batch = make_batch(args.workload, seed=rank, n_curves=args.n_curves)
    pos = batch.positions
    n_curves, n_samples = batch.n_curve, batch.total_samples

    # ---- device-resident arm ------------------------------------------------
    tk = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
    d_arr = (tk(batch.kind, torch.uint8), tk(batch.degree, torch.uint8), tk(batch.dim, torch.uint8),
             tk(batch.knot_off, torch.int64), tk(batch.knots, torch.float64), tk(batch.ctrl_off, torch.int64),
             tk(batch.ctrl, torch.float64))
    d_cnt = tk(batch.n_samples, torch.int32)
    d_pos = tk(pos, torch.float64)
    d_out = torch.empty(n_samples, dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def device_arm(prec, steps, warmup, clocks=False, learned_on=False):
        """Times `steps` table builds + samplings of the resident batch with CUDA
        events (L2 flushed before each); returns the per-step figures."""
        calc = g.ArclengthCalculateGpu.from_device_batch(*d_arr, precision=prec, rtol=batch.rtol, collect_stats=True,
                                                         learned=learned_on)
        if learned_on:
            calc.set_learned_model(model)

        def step():
            if use_graph:
                calc.stepGraph(d_cnt, d_pos, d_out, True, g.GCV_RETURN_US)
            else:
                calc.createArclengthTable()
                calc.arclengthReverseInto(d_cnt, d_pos, d_out, True, g.GCV_RETURN_US)

        for _ in range(warmup):
            step()
        torch.cuda.synchronize()
        launches0 = calc.stats()["n_launches"]
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        r = {"ms_len": [], "ms_samp": [], "ms_setup": [], "n_newton": [], "n_panels": [], "ms_learned": []}
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            for i in range(steps):
                flush.zero_()
                evs[i][0].record()
                step()
                evs[i][1].record()
                st = calc.stats()  # synchronises; outside the events
                r["ms_len"].append(st["ms_length"])
                r["ms_samp"].append(st["ms_sample"])
                r["ms_setup"].append(st["ms_setup"] + st["ms_scan"])
                r["n_newton"].append(st["n_newton"])
                r["n_panels"].append(st["n_panels"])
                r["ms_learned"].append(st["ms_learned"])
            torch.cuda.synchronize()
        if dist:
            dist.barrier()
        total_ms = max_over_ranks(float(sum(x.elapsed_time(y) for x, y in evs)), dist, dev)
        st1 = calc.stats()
        r["launches"] = st1["n_launches"] - launches0
        r["leaves"] = st1["n_leaves"]
        r["deep"] = st1["n_deep_segments"]
        r["ms_per_step"] = total_ms / steps
        r["clocks"] = clk.summary() if clocks else None
        calc.close()
        return r

    use_graph = not args.no_graph
    main_r = device_arm(precision, args.steps, max(args.warmup, 3), clocks=True, learned_on=use_learned)
    plain_r = mixed_r = None
    if precision != g.GCV_PLAIN_FP64 and args.plain_steps > 0:
        plain_r = device_arm(g.GCV_PLAIN_FP64, args.plain_steps, 1)
        if use_learned:
            # the same mixed-precision walk without the network: what the network gains
            mixed_r = device_arm(g.GCV_MIXED, args.plain_steps, 1)
    ms_per_step = main_r["ms_per_step"]
    launches = main_r["launches"]
    leaves = main_r["leaves"]
    ms_samp, n_newton, n_panels = main_r["ms_samp"], main_r["n_newton"], main_r["n_panels"]
    ms_inf = main_r["ms_learned"]
    ms_len = [a - b for a, b in zip(main_r["ms_len"], ms_inf)]  # the length passes without the network
    value = job_throughput(n_curves, ms_per_step, world)
    samples_per_s = world * n_samples / (ms_per_step * 1e-3)

    # ---- accuracy of this run on a subset (vs the oracle) --------------------
    # (reported, not asserted: tests/ carry the parity bars)
    # ---- roofline of the dominant kernel ------------------------------------
    fpe = flops_per_eval(batch)
    samp_flops = float(np.mean(n_newton)) * (8 * (fpe + 4.0) + fpe + 4.0) + n_samples * 20.0
    len_flops = float(np.mean(n_panels)) * (16 * (fpe + 2.0) + 40.0)
    ms_s, ms_l = float(np.mean(ms_samp)), float(np.mean(ms_len))
    fp64_peak = _lib.measure_fma_peak(0)
    fp32_peak = _lib.measure_fma_peak(1)
    if ms_s >= ms_l:
        dom, flops, ms = "k_sample", samp_flops, ms_s
        bytes_alg = n_samples * (8 + 8 + 8) + n_curves * 8
    else:
        dom, flops, ms = "k_length", len_flops, ms_l
        bytes_alg = batch.knots.nbytes + batch.ctrl.nbytes + batch.n_segments.sum() * 8
    achieved = flops / (ms * 1e-3) / 1e12
    peak = fp64_peak if precision == g.GCV_PLAIN_FP64 else fp32_peak
    traffic = None
    prof = os.path.join(ROOT, "profiles", "traffic_per_unit.json")
    if os.path.exists(prof):
        try:
            tpu = json.load(open(prof)).get(f"{dom}:{args.workload}:{args.precision}")
            if tpu:
                traffic = float(tpu) * (n_samples if dom == "k_sample" else float(batch.n_segments.sum()))
        except (ValueError, OSError):
            traffic = None
    hbm_peak = None
    mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(mp):
        hbm_peak = json.load(open(mp)).get("hbm_gbs")
    roofline = {
        "kernel": dom, "bound": "fp64" if precision == g.GCV_PLAIN_FP64 else "fp32",
        "achieved": round(achieved, 4), "peak": round(peak, 4), "unit": "TFLOP/s",
        "frac": round(achieved / peak, 4), "peak_source": "measured in-run by gcv_measure_fma_peak (FMA probe kernel)",
        "traffic": traffic, "ms_per_launch": round(ms, 4), "algorithmic_flops_per_launch": flops,
        "hbm": {"achieved_gbs": round(bytes_alg / (ms * 1e-3) / 1e9, 2), "peak_gbs": hbm_peak,
                "frac": round(bytes_alg / (ms * 1e-3) / 1e9 / hbm_peak, 4) if hbm_peak else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "phases_ms": {"length": round(ms_l, 4), "sample": round(ms_s, 4),
                      "setup_scan": round(float(np.mean(main_r["ms_setup"])), 4),
                      "network_inference": round(float(np.mean(ms_inf)), 4)},
        "work_per_step": {"panels": float(np.mean(n_panels)), "newton_iterations": float(np.mean(n_newton)),
                          "leaves": int(leaves), "segments": int(batch.n_segments.sum()),
                          "length_tflops": round(len_flops / (ms_l * 1e-3) / 1e12, 4),
                          "sample_tflops": round(samp_flops / (ms_s * 1e-3) / 1e12, 4)},
        "fp32_peak_tflops": round(fp32_peak, 2),
    }

    # ---- end-to-end through the public API with host buffers -----------------
    e2e_t, parts = [], []
    h_out = np.zeros(n_samples, np.float64)
    for i in range(max(args.e2e_steps, 1) + 1):
        if dist:
            dist.barrier()
        t = [time.perf_counter()]
        c2 = g.ArclengthCalculateGpu.from_batch(batch, precision=precision, rtol=batch.rtol, learned=use_learned)
        if use_learned:
            c2.set_learned_model(model)
        t.append(time.perf_counter())
        c2.createArclengthTable()
        t.append(time.perf_counter())
        c2.arclengthReverseInto(batch.n_samples, pos, h_out, True, g.GCV_RETURN_US)
        t.append(time.perf_counter())
        c2.close()
        t.append(time.perf_counter())
        if i > 0:
            e2e_t.append(t[-1] - t[0])
            parts.append(np.diff(t) * 1e3)
    e2e_parts = dict(zip(["create", "table", "sample", "destroy"], np.round(np.mean(parts, axis=0), 3).tolist()))
    e2e_s = max_over_ranks(float(np.mean(e2e_t)), dist, dev)
    h2d = batch.nbytes() + batch.n_samples.nbytes + pos.nbytes
    d2h = h_out.nbytes

    # ---- CPU baseline and accuracy (rank 0, N = 1 only) ----------------------
    cpu = acc = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        sub = cpu_sample(batch, args.cpu_sample_curves or auto_cpu_curves(batch, nthreads, 10.0))
        secs, kind = run_cpu_reference(sub, nthreads)
        cpu = {"value": round(sub.n_curve / secs, 3), "unit": "curves/s", "cores": nthreads, "kind": kind,
               "sample": f"{sub.n_curve} curves of the workload ({sub.total_samples} samples), table + sampling, "
                         f"{secs:.2f} s", "samples_per_s": round(sub.total_samples / secs, 1)}
        acc = accuracy_vs_oracle(sub, precision, batch.rtol, model)
    plain = None
    if plain_r is not None:
        pv = job_throughput(n_curves, plain_r["ms_per_step"], world)
        plain = {"value": round(pv, 3), "unit": "curves/s", "ms_per_step": round(plain_r["ms_per_step"], 4),
                 "steps": args.plain_steps, "warmup": 1, "rtol": batch.rtol,
                 "samples_per_s": round(world * n_samples / (plain_r["ms_per_step"] * 1e-3), 1),
                 "phases_ms": {"length": round(float(np.mean(plain_r["ms_len"])), 4),
                               "sample": round(float(np.mean(plain_r["ms_samp"])), 4),
                               "setup_scan": round(float(np.mean(plain_r["ms_setup"])), 4)},
                 "speedup_of_this_form": round(value / pv, 3)}
    gain = None
    if mixed_r is not None:
        mv = job_throughput(n_curves, mixed_r["ms_per_step"], world)
        gain = {"mixed_without_network": {"value": round(mv, 3), "unit": "curves/s",
                                          "ms_per_step": round(mixed_r["ms_per_step"], 4),
                                          "panels": float(np.mean(mixed_r["n_panels"])),
                                          "length_ms": round(float(np.mean(mixed_r["ms_len"])), 4)},
                "with_network": {"panels": float(np.mean(n_panels)), "length_ms": round(float(np.mean(ms_len)), 4),
                                 "inference_ms": round(float(np.mean(ms_inf)), 4)},
                "panels_saved_frac": round(1.0 - float(np.mean(n_panels)) / float(np.mean(mixed_r["n_panels"])), 4),
                "speedup_over_mixed": round(value / mv, 4)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "curves/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if precision == g.GCV_PLAIN_FP64 else ("f32+f64+bf16" if use_learned else "f32+f64"),
            "data": "synthetic: seeded generator (numpy default_rng, seed = rank)",
            "config": {"workload": f"{args.workload}: {WORKLOADS[args.workload][1]}",
                       "precision": args.precision, "rtol": batch.rtol,
                       "curves_per_gpu": n_curves, "samples_per_gpu": n_samples,
                       "l2": "flushed between timed steps (256 MB write, untimed)",
                       "step": "one captured CUDA graph per step (gcv_step_graph)" if use_graph else
                               "createArclengthTable + arclengthReverseInto",
                       "parallelism": f"replicas x{world} (independent curves, no collective)"},
            "samples_per_s": round(samples_per_s, 1),
            "e2e": {"value": round(world * n_curves / e2e_s, 3), "unit": "curves/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "samples_per_s": round(world * n_samples / e2e_s, 1),
                    "ms_per_step": round(e2e_s * 1e3, 3), "breakdown_ms": e2e_parts},
            "gpu_launches": int(launches),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "accuracy_vs_fp64_oracle": acc,
            "plain_fp64_same_batch": plain,
            "learned_gain": gain,
            "clocks": main_r["clocks"],
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def reference_arm(args):
    nthreads = os.cpu_count() or 1
    batch = make_batch(args.workload, seed=0, n_curves=args.n_curves)
    # each step a bounded sample: the whole --steps / --warmup run stays within minutes
    per_step_s = min(5.0, 150.0 / max(args.steps + max(args.warmup, 3), 1))
    sub = cpu_sample(batch, args.cpu_sample_curves or auto_cpu_curves(batch, nthreads, per_step_s))
    times, kind = [], None
    for i in range(max(args.warmup, 3) + args.steps):
        secs, kind = run_cpu_reference(sub, nthreads)
        if i >= max(args.warmup, 3):
            times.append(secs)
    per = float(np.mean(times))
    value = sub.n_curve / per
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "curves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(per * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded generator (numpy default_rng, seed 0)",
        "config": {"workload": f"{args.workload}: {WORKLOADS[args.workload][1]}", "precision": "plain",
                   "sample_curves": sub.n_curve},
        "samples_per_s": round(sub.total_samples / per, 1),
        "cpu_baseline": {"value": round(value, 3), "unit": "curves/s", "cores": nthreads, "kind": kind,
                         "sample": f"{sub.n_curve} curves of the workload ({sub.total_samples} samples) per step, "
                                   "table + sampling, all host threads"},
        "e2e": {"value": round(value, 3), "unit": "curves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
