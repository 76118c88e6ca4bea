"""Benchmark of the SBP-SAT RK4 hot path on GB300.

Workload (one bench "step"): 1000 classical RK4 steps of the 2D first-order
acoustic wave system (u, v, p), rho = K = 1 on [-1,1]^2, N x N = 4096^2 grid
points, SBP order 4, characteristic SAT boundaries, FP64, Gaussian pressure
pulse of width 0.05 at the origin, dt = 0.2 h. Synthetic data.

  value     grid-point stage updates per second (N^2 * 4 stages * 1000 steps
            per bench step), state resident in HBM, whole job over all ranks.
  e2e       the same metric through the C ABI call a user makes (sbp_rk4 with
            a pinned host array: H2D copy, layout packing, 1000 steps,
            unpacking, D2H copy inside the timed region).
  roofline  algorithmic HBM bytes of the fused stage kernel (16*c*s = 384 B per
            point per RK4 step for c = 3 components of s = 8 bytes) divided
            by its measured time, against the measured copy bandwidth.

`--impl reference` times the reference's CPU implementation of the same path
(the reference's own headers when built here as oracle/_ref, else the oracle
restatement) on all host cores, on a bounded sample of the same workload.

Multi-GPU: the path is one grid per device; `--gpus N` runs N independent
replicas (one per rank, launched by torch.distributed.run) and reports the
sum of their throughputs over the slowest rank's time.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "hpc-reading-course_gb300")
sys.path.insert(0, os.path.join(PKG, "python"))
sys.path.insert(0, PKG)
import fields  # noqa: E402  (seeded inputs: initial data and coefficient fields)

METRIC = "RK4 point-updates/s"
# The port's speed against the reference's own wave_hom RHS headers, both built with the
# reference's -O3 -ffast-math, one thread, 1024^2, orders 2/4/6 (oracle/time_reference.py,
# on the x86 host where the reference checkout exists; the GPU machine has none).
REF_CODE_RATIO = "port / reference code = 1.01 / 0.94 / 0.91 (orders 2 / 4 / 6)"
UNIT = "grid-point stage updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--grid", type=int, default=4096)
    ap.add_argument("--order", type=int, default=4, choices=[2, 4, 6])
    ap.add_argument("--rk-steps", type=int, default=1000)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--bc", default="characteristic", choices=["characteristic", "free_surface"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the forms record (other orders and sizes, FP32, the batched form)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--study", default=None,
                    choices=["precision", "batched", "learned", "rk45", "wave3d", "decomp", "cnn"],
                    help="precision: variable rho, K (seeded Fourier fields) to --t-end in FP64 and in "
                         "compensated FP32; prints errors of FP32 against FP64 and both wall times. "
                         "batched: 512 uneven wave/advection instances in one batch, FP64 and FP32. "
                         "rk45: adaptive RKF45 (ts_rk45) on the bench's wave problem to --rk45-t-end. "
                         "wave3d: the 3D wave system on --grid3d^3 points, FP64 and FP32")
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--batched-forms", default="fp64,fp32", help="batched: comma-separated precisions to run")
    ap.add_argument("--no-entry-sweep", action="store_true",
                    help="batched: skip timing every group on each configuration-table entry")
    ap.add_argument("--no-one-by-one", action="store_true",
                    help="batched: skip the same instances run one after another through single contexts")
    ap.add_argument("--trajectories", type=int, default=2000, help="learned: training trajectories")
    ap.add_argument("--epochs", type=int, default=30, help="learned: training epochs per round")
    ap.add_argument("--rollout-rounds", type=int, default=2,
                    help="learned: rounds of training on windows started on the corrected solve's states")
    ap.add_argument("--t-end", type=float, default=1.0)
    ap.add_argument("--rk45-t-end", type=float, default=0.25, help="rk45: final time")
    ap.add_argument("--grid3d", type=int, default=256, help="wave3d: points per direction")
    ap.add_argument("--decomps", default="1x1,2x2,4x4,8x8", help="decomp: the px x py decompositions to run")
    return ap.parse_args()


def initial_state(n: int):
    """Gaussian pressure pulse exp(-(x^2+y^2)/0.05^2), u = v = 0, AoS (j, i, comp)."""
    return fields.gaussian_pulse(n, n, 0.0, 0.0, 0.05, 1.0)


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [s.strip() for s in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_summary(order: int, precision: str) -> str:
    """The committed ncu summary of the stage kernel this precision runs."""
    kernel = "wave_fixed" if precision == "fp64" else "wave_stage"
    return os.path.join("profiles", f"{kernel}_{precision}_o{order}_4096.md")


def profiled_traffic(order: int, precision: str):
    """DRAM bytes per point of one middle-stage launch, from the committed ncu summary, if any."""
    path = os.path.join(ROOT, profile_summary(order, precision))
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("| traffic_bytes_per_point_stage |"):
                    return float(line.split("|")[2].split()[0])
    except (OSError, ValueError, IndexError):
        pass
    return None


def cpu_baseline(n: int, order: int, precision: str, bc: str, budget_s: float, repeats: int = 1):
    """The path on the host cores: the oracle restatement of the reference's
    operators (oracle/sbp_oracle.c, pinned bit for bit to the reference's own
    headers by tests/test_oracle.py), built with the reference's -O3
    -ffast-math and run with OpenMP over all cores, on the same problem as the
    GPU arm (rho = K = 1, the same SAT). oracle/_ref, the reference's headers
    compiled in this checkout, is built only where the reference checkout
    exists and is not timed here. Returns (rates, kind, threads, sample)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    port = O.Port(O.PORT_OPT_SO)  # built with the reference's -O3 -ffast-math
    threads = os.cpu_count() or 1
    port.set_threads(threads)
    v = initial_state(n)
    h = 2.0 / (n - 1)
    pb = O.Problem(O.WAVE_HOM_2D, order, n, n,
                   bc=O.BC_CHARACTERISTIC if bc == "characteristic" else O.BC_REFERENCE)
    t0 = time.perf_counter()
    v = port.rk4(pb, v, 0.0, 0.2 * h, 1)
    t1 = time.perf_counter() - t0
    steps = max(1, min(1000, int(budget_s / max(t1, 1e-6))))
    rates = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        v = port.rk4(pb, v, 0.0, 0.2 * h, steps)
        el = time.perf_counter() - t0
        rates.append(n * n * 4 * steps / el)
    kind = "port"
    sample = (f"{steps} RK4 steps of the {n}x{n} order-{order} FP64 wave workload "
              f"({'characteristic' if bc == 'characteristic' else 'free-surface'} SAT), oracle restatement "
              f"(oracle/sbp_oracle.c with the reference's -O3 -ffast-math, OpenMP) on {threads} threads")
    return rates, kind, threads, sample


def max_over_ranks(value: float, dist, device: str) -> float:
    """The largest of every rank's `value` (an all_reduce MAX on `device`, which the
    process group's backend must reach); `value` itself without a process group."""
    if not dist:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank: int):
    if rank != 0:
        return
    budget = 3.0
    rates, kind, threads, sample = cpu_baseline(args.grid, args.order, args.precision, args.bc, budget,
                                                repeats=args.warmup + args.steps)
    timed = rates[args.warmup:]
    value = statistics.median(timed)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample,
                         "port_vs_reference_code": REF_CODE_RATIO},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_of(args):
    return {"workload": f"2D acoustic wave (u,v,p), rho=K=1, {args.grid}x{args.grid}, SBP order {args.order}, "
                        f"{args.bc} SAT, {args.precision.upper()}, Gaussian pulse w=0.05, dt=0.2h, "
                        f"{args.rk_steps} RK4 steps per bench step",
            "grid": [args.grid, args.grid], "order": args.order, "rk4_steps_per_step": args.rk_steps,
            "precision": args.precision, "bc": args.bc,
            "l2_flush": f"inputs larger than L2: {args.grid * args.grid * 3 * (8 if args.precision == 'fp64' else 4) / 1e6:.0f}"
                        " MB per state vector, 4 state vectors",
            "parallelism": f"replicas x{args.gpus}"}


def run_precision_study(args):
    """Variable rho, K = 1 + 0.5 tanh(8 seeded Fourier modes, |k| <= 6) (seeds 0, 1), pulse at the
    origin, characteristic SAT, CFL 0.2 on the largest wave speed, to t_end: FP32 (compensated) vs FP64."""
    import numpy as np
    import torch

    import build as gpu_build
    import fields
    import sbpgpu

    gpu_build.build()
    n, order = args.grid, args.order
    rho, K = fields.fourier_field(n, 0), fields.fourier_field(n, 1)
    h = 2.0 / (n - 1)
    cmax = float(np.sqrt((K / rho).max()))
    nsteps, dt = sbpgpu.rk4_nsteps(args.t_end, 0.2 * h / cmax)
    v0 = fields.gaussian_pulse(n, n)
    out, times = {}, {}
    for name, prec in (("fp64", sbpgpu.FP64), ("fp32", sbpgpu.FP32)):
        with sbpgpu.Context(sbpgpu.WAVE_VAR_2D, order, n, n, bc=sbpgpu.BC_CHARACTERISTIC, precision=prec,
                            rho=rho, K=K) as ctx:
            ctx.set_state(v0)
            ctx.step_resident(0.0, dt, 3)  # warm-up (graph capture), then restart from v0
            ctx.synchronize()
            ctx.set_state(v0)
            ctx.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            stream = torch.cuda.ExternalStream(ctx.stream)
            ev0.record(stream)
            ctx.step_resident(0.0, dt, nsteps)
            ev1.record(stream)
            ctx.synchronize()
            times[name] = ev0.elapsed_time(ev1) / 1e3
            out[name] = ctx.get_state()
    d = out["fp32"] - out["fp64"]
    l2 = float(np.sqrt(h * h * np.sum(d * d)))
    ref_l2 = float(np.sqrt(h * h * np.sum(out["fp64"] ** 2)))
    line = {"study": "precision", "grid": [n, n], "order": order, "t_end": args.t_end, "steps": nsteps, "dt": dt,
            "rho_range": [float(rho.min()), float(rho.max())], "K_range": [float(K.min()), float(K.max())],
            "fp32_vs_fp64": {"l2": l2, "l2_rel": l2 / ref_l2, "max": float(np.abs(d).max()),
                             "max_rel": float(np.abs(d).max() / np.abs(out["fp64"]).max())},
            "seconds": times, "speedup_fp32": times["fp64"] / times["fp32"],
            "fields": "1 + 0.5 tanh(sum of 8 Fourier modes, |k| <= 6, A ~ N(0,1)), seeds 0 (rho) and 1 (K)"}
    # against an exact solution: the standing mode (n, m) = (3, 4) of the rho = K = 1 system with
    # free-surface SAT, both precisions to t = 0.05 on grids from 512^2 to the study's grid, the L2
    # error (sqrt(hx hy) ||v - v_exact||) and the wall time of each
    t_exact = 0.05
    rows = []
    for ng in sorted({512, 1024, 2048, n}):
        if ng > n:
            continue
        hg = 2.0 / (ng - 1)
        ns, dts = sbpgpu.rk4_nsteps(t_exact, 0.2 * hg)
        exact = fields.standing_mode(ng, ng, t_exact)
        ex = {"grid": ng, "steps": ns}
        for name, prec in (("fp64", sbpgpu.FP64), ("fp32", sbpgpu.FP32)):
            with sbpgpu.Context(sbpgpu.WAVE_HOM_2D, order, ng, ng, precision=prec) as ctx:
                ctx.set_state(fields.standing_mode(ng, ng, 0.0))
                ctx.step_resident(0.0, dts, 3)  # warm-up (graph capture), then restart
                ctx.synchronize()
                ctx.set_state(fields.standing_mode(ng, ng, 0.0))
                ctx.synchronize()
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                stream = torch.cuda.ExternalStream(ctx.stream)
                ev0.record(stream)
                ctx.step_resident(0.0, dts, ns)
                ev1.record(stream)
                ctx.synchronize()
                l2, _ = ctx.error_norms(exact)
                ex[name] = {"l2_error": l2, "seconds": ev0.elapsed_time(ev1) / 1e3}
        ex["error_ratio_fp32_fp64"] = ex["fp32"]["l2_error"] / ex["fp64"]["l2_error"]
        ex["speedup_fp32"] = ex["fp64"]["seconds"] / ex["fp32"]["seconds"]
        rows.append(ex)
    line2 = {"study": "precision_exact", "order": order, "problem": "wave_hom standing mode (3, 4)",
             "bc": "free surface", "t_end": t_exact, "dt": "0.2 h", "grids": rows}
    print(json.dumps(line), flush=True)
    print(json.dumps(line2), flush=True)


def _timed_steps(ctx, dt: float, steps: int) -> float:
    """Seconds of `steps` resident RK4 steps, CUDA events on the context's stream."""
    import torch

    stream = torch.cuda.ExternalStream(ctx.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    ctx.step_resident(0.0, dt, steps)
    ev1.record(stream)
    ctx.synchronize()
    return ev0.elapsed_time(ev1) / 1e3


def _relerr(a, b) -> float:
    import numpy as np

    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def measure_forms(peak: float, device: int = 0) -> dict:
    """The bench's other forms, each bounded to seconds, for the JSON line's `forms` record:
    FP64 at orders 2 and 6 (4096^2) and at 1024^2 (order 4); FP32 at 4096^2 with its error
    against FP64 after the same steps; the 512-instance batch in FP64 and FP32 with the largest
    relative error of 16 sampled instances against the plain FP64 path (single contexts).
    Roofline fractions use the same algorithmic bytes as the headline: 16*c*s per point per
    RK4 step (19*c*4 for compensated FP32)."""
    import numpy as np
    import torch

    import sbpgpu

    out = {}
    bc = sbpgpu.BC_CHARACTERISTIC
    for name, n, order, steps in (("fp64_4096_o2", 4096, 2, 200), ("fp64_4096_o6", 4096, 6, 200),
                                  ("fp64_1024_o4", 1024, 4, 1000)):
        dt = 0.2 * 2.0 / (n - 1)
        with sbpgpu.Context(sbpgpu.WAVE_HOM_2D, order, n, n, bc=bc, device=device) as c:
            c.set_state(initial_state(n))
            c.step_resident(0.0, dt, 50)
            c.synchronize()
            sec = _timed_steps(c, dt, steps)
        rate = n * n * 4 * steps / sec
        out[name] = {"value": rate, "unit": UNIT, "rk4_steps": steps, "roofline_frac": rate * 96 / 1e9 / peak}
    # FP32 against FP64 from the same state after the same steps
    n, order, steps = 4096, 4, 500
    dt = 0.2 * 2.0 / (n - 1)
    v0 = initial_state(n)
    res = {}
    for prec in (sbpgpu.FP64, sbpgpu.FP32):
        with sbpgpu.Context(sbpgpu.WAVE_HOM_2D, order, n, n, bc=bc, precision=prec, device=device) as c:
            c.set_state(v0)
            c.step_resident(0.0, dt, 3)  # graph capture, then restart from v0
            c.synchronize()
            c.set_state(v0)
            sec = _timed_steps(c, dt, steps)
            res[prec] = (sec, c.get_state())
    rate = n * n * 4 * steps / res[sbpgpu.FP32][0]
    d = res[sbpgpu.FP32][1] - res[sbpgpu.FP64][1]
    out["fp32_4096_o4"] = {"value": rate, "unit": UNIT, "rk4_steps": steps,
                           "roofline_frac": rate * 57 / 1e9 / peak,
                           "fp64_seconds_same_steps": res[sbpgpu.FP64][0], "fp32_seconds": res[sbpgpu.FP32][0],
                           "rel_max_err_vs_fp64": _relerr(res[sbpgpu.FP32][1], res[sbpgpu.FP64][1]),
                           "rel_l2_err_vs_fp64": float(np.linalg.norm(d) / np.linalg.norm(res[sbpgpu.FP64][1]))}
    # the batched form
    insts, states = fields.batched_instances(512)
    sample = fields.batched_sample(insts, 16)
    acc_steps = 100
    plain = {}
    for k in sample:
        d = insts[k]
        if d["problem"] == sbpgpu.WAVE_HOM_2D:
            ones = np.ones(d["nx"] * d["ny"])
            c = sbpgpu.Context(sbpgpu.WAVE_VAR_2D, d["order"], d["nx"], d["ny"], rho=ones, K=ones * d["c"] ** 2,
                               bc=d["bc"], device=device)
        else:
            c = sbpgpu.Context(sbpgpu.ADVECTION_2D, d["order"], d["nx"], d["ny"], a=d["a"], b=d["b"], device=device)
        with c:
            plain[k] = c.rk4(states[k], 0.0, d["dt"], acc_steps)
    cache = os.environ.get("SBP_TUNE_CACHE", os.path.join(PKG, "_build", "batch_tiles.json"))
    for pname, prec, es, comp in (("batched_fp64", sbpgpu.FP64, 8, 16), ("batched_fp32", sbpgpu.FP32, 4, 19)):
        with sbpgpu.Batch(insts, precision=prec, device=device) as b:
            for k, v in enumerate(states):
                b.set_state(k, v)
            b.autotune(cache)
            cfgs = batch_kernel_configs(b, sbpgpu)
            b.step_resident(acc_steps)
            b.synchronize()
            err = max(_relerr(b.get_state(k), plain[k]) for k in sample)
            b.step_resident(100)  # warm
            b.synchronize()
            stream = torch.cuda.ExternalStream(b.stream)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            b.step_resident(200)
            ev1.record(stream)
            b.synchronize()
            sec = ev0.elapsed_time(ev1) / 1e3
            pts = b.points
        comps = sum((3 if d["problem"] == sbpgpu.WAVE_HOM_2D else 1) * d["nx"] * d["ny"] for d in insts)
        bytes_per_step = comp * es * comps  # per RK4 step, all instances
        out[pname] = {"value": pts * 4 * 200 / sec, "unit": UNIT, "instances": len(insts), "points": pts,
                      "rk4_steps": 200, "roofline_frac": bytes_per_step * 200 / sec / 1e9 / peak,
                      "max_rel_err_vs_plain_fp64": err, "sampled_instances": len(sample),
                      "error_after_rk4_steps": acc_steps, "kernel_configs": cfgs}
    return out


def batch_kernel_configs(b, sbpgpu):
    """The kernel configuration each (problem, order) group of a batch runs: tile rows, compute
    warps, ring depth, CTAs per SM."""
    out = {}
    for name, problem in (("wave", sbpgpu.WAVE_HOM_2D), ("advection", sbpgpu.ADVECTION_2D)):
        for order in (2, 4, 6):
            cfg = b.kernel_config(order, problem)
            if cfg["rows"]:
                out[f"{name}_o{order}"] = [cfg["rows"], cfg["warps"], cfg["ring"], cfg["ctas_per_sm"]] + (
                    ["fixed-point"] if cfg["converters"] else [])
    return out


def run_batched_study(args):
    """One batch of --instances uneven instances; 100-step graph chunks; autotuned kernel
    configurations ([tile rows, compute warps, ring depth, CTAs per SM] per group)."""
    import torch

    import build as gpu_build
    import sbpgpu

    gpu_build.build()
    insts, states = fields.batched_instances(args.instances)
    cache = os.environ.get("SBP_TUNE_CACHE", os.path.join(PKG, "_build", "batch_tiles.json"))
    out = {"study": "batched", "instances": len(insts),
           "waves": sum(1 for d in insts if d["problem"] == sbpgpu.WAVE_HOM_2D),
           "orders": {o: sum(1 for d in insts if d["order"] == o) for o in (2, 4, 6)}}
    forms = [f for f in (("fp64", sbpgpu.FP64), ("fp32", sbpgpu.FP32)) if f[0] in args.batched_forms.split(",")]
    for name, prec in forms:
        with sbpgpu.Batch(insts, precision=prec) as b:
            for k, v in enumerate(states):
                b.set_state(k, v)
            b.autotune(cache)
            stream = torch.cuda.ExternalStream(b.stream)
            b.step_resident(100)  # warm-up: graph capture
            b.synchronize()
            launches0 = b.launches
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            chunks = max(1, args.steps)
            ev0.record(stream)
            b.step_resident(100 * chunks)
            ev1.record(stream)
            b.synchronize()
            sec = ev0.elapsed_time(ev1) / 1e3
            units = b.points * 4 * 100 * chunks
            out[name] = {"value": units / sec, "unit": UNIT, "seconds": sec, "rk4_steps": 100 * chunks,
                         "points": b.points, "kernel_configs": batch_kernel_configs(b, sbpgpu),
                         "gpu_launches": b.launches - launches0}
            # every group on the same table entry, entry by entry (the autotuner's choices per
            # group above; this shows what each axis gives on the whole batch)
            per_entry = []
            for index in range(0 if args.no_entry_sweep else 4):
                for order in (2, 4, 6):
                    for problem in (sbpgpu.WAVE_HOM_2D, sbpgpu.ADVECTION_2D):
                        b.select_config(order, problem, index)
                b.step_resident(100)  # graph capture
                b.synchronize()
                ev0.record(stream)
                b.step_resident(100 * chunks)
                ev1.record(stream)
                b.synchronize()
                per_entry.append({"entry": index, "value": units / (ev0.elapsed_time(ev1) / 1e3),
                                  "kernel_configs": batch_kernel_configs(b, sbpgpu)})
            if per_entry:
                out[name]["every_group_on_entry"] = per_entry
    # the same instances one after another through single contexts (waves with c != 1 through the
    # variable-coefficient context, rho = 1, K = c^2), the same number of RK4 steps; creation and
    # graph capture outside the timed region
    import numpy as np

    steps = 100 * max(1, args.steps)
    for name, prec in forms if not args.no_one_by_one else ():
        ctxs = []
        for d, v in zip(insts, states):
            if d["problem"] == sbpgpu.WAVE_HOM_2D:
                ones = np.ones(d["nx"] * d["ny"])
                c = sbpgpu.Context(sbpgpu.WAVE_VAR_2D, d["order"], d["nx"], d["ny"], rho=ones, K=ones * d["c"] ** 2,
                                   bc=d["bc"], precision=prec)
            else:
                c = sbpgpu.Context(sbpgpu.ADVECTION_2D, d["order"], d["nx"], d["ny"], a=d["a"], b=d["b"],
                                   precision=prec)
            c.set_state(v)
            c.step_resident(0.0, d["dt"], 50)  # warm-up: graph capture
            c.synchronize()
            ctxs.append(c)
        device = 0.0
        t0 = time.perf_counter()
        for c, d in zip(ctxs, insts):
            stream = torch.cuda.ExternalStream(c.stream)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            c.step_resident(0.0, d["dt"], steps)
            ev1.record(stream)
            c.synchronize()
            device += ev0.elapsed_time(ev1) / 1e3
        wall = time.perf_counter() - t0
        for c in ctxs:
            c.close()
        out[name]["one_by_one"] = {"device_seconds": device, "wall_seconds": wall,
                                   "speedup_batched_device": device / out[name]["seconds"],
                                   "speedup_batched_wall": wall / out[name]["seconds"]}
    out["tune_cache"] = cache
    print(json.dumps(out), flush=True)


def run_rk45_study(args):
    """Adaptive RKF45 (the reference's ts_rk45: PETSc TSRK5F + TSADAPTBASIC) on the bench's
    problem: 2D wave, rho = K = 1, characteristic SAT, Gaussian pulse w = 0.05 at the origin,
    --grid^2 points, order --order, FP64, default tolerances (atol = rtol = 1e-4), dt0 = 0.2 h,
    from t = 0 to --rk45-t-end. Reports the attempts, the wall time (host loop included), RHS
    point-evaluations/s and the bytes an attempt moves against measured HBM bandwidth; beside it
    fixed-step RK4 at dt = 0.2 h over the same interval, and the oracle's restatement on all host
    cores for a bounded number of attempts of the same run (its step limit)."""
    import numpy as np

    import build as gpu_build
    import sbpgpu

    gpu_build.build()
    n, order, t_end = args.grid, args.order, args.rk45_t_end
    h = 2.0 / (n - 1)
    v0 = initial_state(n)
    with sbpgpu.Context(sbpgpu.WAVE_HOM_2D, order, n, n, bc=sbpgpu.BC_CHARACTERISTIC) as ctx:
        ctx.set_state(v0)
        ctx.rk45_resident(0.0, 4 * 0.2 * h, 0.2 * h)  # warm-up: graph capture
        ctx.set_state(v0)
        ctx.synchronize()
        t0 = time.perf_counter()
        st = ctx.rk45_resident(0.0, t_end, 0.2 * h)
        t_rk45 = time.perf_counter() - t0
        nsteps, dt = sbpgpu.rk4_nsteps(t_end, 0.2 * h)
        ctx.set_state(v0)
        ctx.step_resident(0.0, dt, 2)  # warm-up
        ctx.set_state(v0)
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.step_resident(0.0, dt, nsteps)
        ctx.synchronize()
        t_rk4 = time.perf_counter() - t0
    attempts = st["accepted"] + st["rejected"]
    evals = 6.0 * n * n * attempts
    # state vectors moved per point and attempt by the fused wave stages: stage 1 reads u and
    # writes k1, w2; stage s = 2..5 reads w_s, u, k_1..k_{s-1} and writes k_s, w_{s+1}; stage 6
    # reads w6, u, k1, k3, k4, k5 and writes the candidate; an accepted attempt copies it to u
    vectors = 3 + sum(s + 3 for s in range(2, 6)) + 7 + 2.0 * st["accepted"] / max(attempts, 1)
    bytes_attempt = vectors * 3 * 8 * n * n
    peak, src = measured_peaks()
    line = {"study": "rk45", "grid": [n, n], "order": order, "t_end": t_end, "dt0": 0.2 * h,
            "tolerances": {"atol": 1e-4, "rtol": 1e-4}, "accepted": st["accepted"], "rejected": st["rejected"],
            "dt_last": st["dt_next"], "seconds": t_rk45, "rhs_point_evals_per_s": evals / t_rk45,
            "bytes_per_point_attempt": vectors * 24,
            "achieved_gbs": bytes_attempt * attempts / t_rk45 / 1e9, "peak_gbs": peak, "peak_source": src,
            "frac": bytes_attempt * attempts / t_rk45 / 1e9 / peak,
            "rk4_fixed": {"dt": dt, "steps": nsteps, "seconds": t_rk4}}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        O.build()
        port = O.Port(O.PORT_OPT_SO)
        threads = os.cpu_count() or 1
        port.set_threads(threads)
        ones = np.ones(n * n)
        pb = O.Problem(O.WAVE_VAR_2D, order, n, n, rho=ones, K=ones, bc=O.BC_CHARACTERISTIC)
        k = max(1, min(attempts, 8))
        t0 = time.perf_counter()
        _, cst = port.rk45(pb, v0, 0.0, t_end, 0.2 * h, max_steps=k)
        t_cpu = time.perf_counter() - t0
        done = cst["accepted"] + cst["rejected"]
        line["cpu"] = {"rhs_point_evals_per_s": 6.0 * n * n * done / t_cpu, "attempts": done, "seconds": t_cpu,
                       "cores": threads, "kind": "port",
                       "sample": f"the first {done} attempts of the same run (oracle step limit)"}
    print(json.dumps(line), flush=True)


def run_decomp_study(args):
    """The decomposed path (sbp_decomp_*): the --grid^2 wave (rho = K = 1, order --order, FP64,
    characteristic SAT, Gaussian pulse) as px x py subdomains (--decomps) with ghost lines, the halo
    exchange fused into the stage kernels, against the single-grid context; 50 RK4 steps each after
    3 warm-up steps, wall time around the synchronous calls, and the two results compared."""
    import numpy as np

    import build as gpu_build
    import sbpgpu

    gpu_build.build()
    n, order, steps = args.grid, args.order, 50
    h = 2.0 / (n - 1)
    dt = 0.2 * h
    v0 = initial_state(n)
    out = {"study": "decomp", "grid": [n, n], "order": order, "rk4_steps": steps, "bc": "characteristic"}
    with sbpgpu.Context(sbpgpu.WAVE_HOM_2D, order, n, n, bc=sbpgpu.BC_CHARACTERISTIC) as c:
        c.set_state(v0)
        c.step_resident(0.0, dt, steps)  # warm-up: captures the step graphs
        c.set_state(v0)
        c.step_resident(0.0, dt, 3)
        c.synchronize()
        t0 = time.perf_counter()
        c.step_resident(0.0, dt, steps)
        c.synchronize()
        sec = time.perf_counter() - t0
        single = c.get_state()
    out["single_grid"] = {"point_stage_per_s": 4.0 * n * n * steps / sec, "seconds": sec}
    rows = []
    for px, py in (tuple(int(v) for v in d.split("x")) for d in args.decomps.split(",")):
        with sbpgpu.Decomp(order, n, n, px, py, bc=sbpgpu.BC_CHARACTERISTIC) as d:
            d.set_state(v0)
            d.step_resident(dt, steps)  # warm-up: captures the step graph
            d.set_state(v0)
            d.step_resident(dt, 3)
            t0 = time.perf_counter()
            d.step_resident(dt, steps)
            sec = time.perf_counter() - t0
            got = d.get_state()
        rows.append({"px": px, "py": py, "point_stage_per_s": 4.0 * n * n * steps / sec, "seconds": sec,
                     "rel_max_diff_vs_single": float(np.max(np.abs(got - single)) / np.max(np.abs(single)))})
    out["decomposed"] = rows
    print(json.dumps(out), flush=True)


def run_wave3d_study(args):
    """3D wave (u, v, w, p), rho = K = 1, characteristic SAT on the six faces, Gaussian pulse
    w = 0.2 at the origin, --grid3d^3 points, order --order, dt = 0.2 h, 100 RK4 steps per timed run,
    FP64 and compensated FP32, state resident in HBM, timed with CUDA events on the context's stream.
    Roofs: HBM with 16 c s bytes per point and RK4 step (c = 4), and for FP64 the FP64 pipe at
    about 33 FP64 instructions per point-stage (order 4: six derivatives of 4 instructions, two adds,
    7 for the stage update on average). CPU: the oracle restatement on all host cores, a bounded
    number of steps."""
    import numpy as np
    import torch

    import build as gpu_build
    import sbpgpu

    gpu_build.build()
    n, order, steps = args.grid3d, args.order, 100
    h = 2.0 / (n - 1)
    dt = 0.2 * h
    x = np.linspace(-1, 1, n)
    v0 = np.zeros((n, n, n, 4))
    v0[..., 3] = np.exp(-(x[None, None, :] ** 2 + x[None, :, None] ** 2 + x[:, None, None] ** 2) / 0.2**2)
    v0 = v0.ravel()
    peak, src = measured_peaks()
    dfma = sbpgpu.probe_dfma_rate() if hasattr(sbpgpu, "probe_dfma_rate") else None
    out = {"study": "wave3d", "grid": [n, n, n], "order": order, "rk4_steps": steps, "dt": dt,
           "bc": "characteristic", "peak_gbs": peak, "peak_source": src}
    for name, prec, s in (("fp64", sbpgpu.FP64, 8), ("fp32", sbpgpu.FP32, 4)):
        with sbpgpu.Context(sbpgpu.WAVE_3D, order, n, n, n, bc=sbpgpu.BC_CHARACTERISTIC, precision=prec) as ctx:
            ctx.set_state(v0)
            ctx.step_resident(0.0, dt, 3)  # warm-up (graph capture)
            ctx.synchronize()
            stream = torch.cuda.ExternalStream(ctx.stream)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            ctx.step_resident(0.0, dt, steps)
            ev1.record(stream)
            ctx.synchronize()
            sec = ev0.elapsed_time(ev1) / 1e3
        rate = 4.0 * n**3 * steps / sec
        bytes_step = (16 * 4 * s + (2 * 4 * s if prec == sbpgpu.FP32 else 0)) * n**3
        line = {"point_stage_per_s": rate, "seconds": sec, "achieved_gbs": bytes_step * steps / sec / 1e9}
        line["hbm_frac"] = line["achieved_gbs"] / peak
        if prec == sbpgpu.FP64 and dfma:
            line["fp64_alu_bound_point_stage_per_s"] = dfma / 33.0
            line["fp64_alu_frac"] = rate / (dfma / 33.0)
        out[name] = line
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        O.build()
        port = O.Port(O.PORT_OPT_SO)
        threads = os.cpu_count() or 1
        port.set_threads(threads)
        pb = O.Problem(O.WAVE_3D, order, n, n, n, bc=O.BC_CHARACTERISTIC)
        t0 = time.perf_counter()
        port.rk4(pb, v0, 0.0, dt, 1)
        t1 = time.perf_counter() - t0
        k = max(1, min(steps, int(10.0 / max(t1, 1e-6))))
        t0 = time.perf_counter()
        port.rk4(pb, v0, 0.0, dt, k)
        sec = time.perf_counter() - t0
        out["cpu"] = {"point_stage_per_s": 4.0 * n**3 * k / sec, "cores": threads, "kind": "port",
                      "sample": f"{k} RK4 steps of the same run"}
    print(json.dumps(out), flush=True)


def run_learned_study(args):
    """Two-layer problem (rho, K x4 across y = 0): coarse 257 x 2*129 order-4 solve corrected by the
    network every 4 steps, trained on restricted fine (1025 x 2*513, FP64) trajectories with seeded
    pulse position U[-0.5,0.5]^2, width U[0.02,0.1], amplitude U[0.5,2] (seeds 1000..), two windows
    drawn from the 16-window horizon per trajectory, started on the restricted fine state; then
    `--rollout-rounds` rounds that add windows started on the corrected solve's own states. Measured
    against the fine solve on 100 held-out trajectories (seeds 5000..5099) after 16 windows, and every
    form, the fine one included, against a solve at twice the fine resolution ("vs_truth")."""
    import numpy as np
    import torch

    import build as gpu_build
    import learned
    import sbpgpu

    gpu_build.build()
    s = learned.Setup()
    sv = learned.Solvers(s, mid=True, truth=True)
    t0 = time.perf_counter()
    seeds = range(1000, 1000 + args.trajectories)
    X, Y, scales = learned.normalize(*learned.collect(sv, seeds, 16, keep=2))
    t_data = time.perf_counter() - t0
    t_train = 0.0
    rounds = []
    with sbpgpu.Cnn(2 * s.nbc, s.nxc, 8, stream=sv.stream.cuda_stream) as net:
        for r in range(1 + args.rollout_rounds):
            if r > 0:  # windows started on the corrected solve's own states
                t0 = time.perf_counter()
                X2, Y2, _ = learned.normalize(*learned.collect(sv, seeds, 16, keep=2,
                                                               solver=learned.LearnedSolver(sv, net, scales)),
                                              scales)
                X, Y = torch.cat([X, X2]), torch.cat([Y, Y2])
                del X2, Y2
                t_data += time.perf_counter() - t0
            t0 = time.perf_counter()
            losses = learned.train(net, X, Y, epochs=args.epochs, batch=8, lr=1e-3, seed=r)
            torch.cuda.synchronize()
            t_train += time.perf_counter() - t0
            rounds.append({"samples": int(X.shape[0]), "loss_first": float(np.mean(losses[:20])),
                           "loss_last": float(np.mean(losses[-20:]))})
        n_samples = int(X.shape[0])
        del X, Y
        solver = learned.LearnedSolver(sv, net, scales)
        res = learned.evaluate(sv, solver, range(5000, 5100), windows=16)
    out = {"study": "learned", "coarse_grid": [s.nxc, 2 * s.nbc], "fine_grid": [s.nxf, 2 * s.nbf],
           "params": sbpgpu.Cnn.param_count(), "trajectories": args.trajectories, "training_samples": n_samples,
           "epochs_per_round": args.epochs, "rounds": rounds,
           "loss_zero_correction": 1.0, "seconds_data": t_data, "seconds_train": t_train,
           "eval_windows": 16, "eval_t_end": 16 * s.window * s.dtc,
           "rel_l2_coarse": float(np.mean(res["coarse"])), "rel_l2_learned": float(np.mean(res["learned"])),
           "rel_l2_coarse_median": float(np.median(res["coarse"])),
           "rel_l2_learned_median": float(np.median(res["learned"])),
           "learned_better": int(np.sum(np.array(res["learned"]) < np.array(res["coarse"]))),
           "mid_grid": [2 * s.nxc - 1, 2 * (2 * s.nbc - 1)], "rel_l2_mid": float(np.mean(res["mid"])),
           "rel_l2_mid_median": float(np.median(res["mid"])),
           "seconds_fine": res["t_fine"], "seconds_coarse": res["t_coarse"], "seconds_learned": res["t_learned"],
           "seconds_mid": res["t_mid"],
           "vs_truth": {"truth_grid": [sv.truth_shape[0], 2 * sv.truth_shape[1]],
                        **{k: float(np.mean(v)) for k, v in res["vs_truth"].items()},
                        **{k + "_median": float(np.median(v)) for k, v in res["vs_truth"].items()},
                        "learned_over_fine": float(np.mean(res["vs_truth"]["learned"]) /
                                                   np.mean(res["vs_truth"]["fine"])),
                        "fine_seconds_over_learned": res["t_fine"] / res["t_learned"]},
           "fallbacks": solver.fallbacks, "held_out": 100}
    print(json.dumps(out), flush=True)


def run_cnn_study(args):
    """The learned correction's network at the learned study's shape (8 images of 258 x 257, the
    coarse two-layer grid): one forward pass, and one training step (forward, loss, weight, bias and
    input gradients, Adam), random inputs, CUDA events on the network's stream after warm-up. FLOPs:
    2 * 9 * cin * cout per pixel and convolution (padded channels 32, 32, 32, 32 -> 32, 32, 32, 16);
    a training step adds the input gradients of layers 1-3 and the four weight gradients."""
    import numpy as np
    import torch

    import build as gpu_build
    import sbpgpu

    gpu_build.build()
    B, H, W = 8, 258, 257
    rng = np.random.default_rng(11)
    x = torch.from_numpy(rng.standard_normal((B, H, W, 24)).astype(np.float32)).cuda()
    t = torch.from_numpy((0.1 * rng.standard_normal((B, H, W, 3))).astype(np.float32)).cuda()
    out = torch.empty((B, H, W, 3), dtype=torch.float32, device="cuda")
    P = B * H * W
    convs = [(32, 32), (32, 32), (32, 32), (32, 16)]
    fwd_flops = sum(2 * 9 * ci * co for ci, co in convs) * P
    train_flops = fwd_flops + sum(2 * 9 * ci * co for ci, co in convs[1:]) * P + fwd_flops
    peak = measured_peaks_tensor()
    res = {"study": "cnn", "batch": B, "height": H, "width": W}
    stream = torch.cuda.current_stream()
    with sbpgpu.Cnn(H, W, B, stream=stream.cuda_stream) as net:  # on torch's stream: the events below see it
        for _ in range(3):
            net.forward(x.data_ptr(), B, out.data_ptr())
            net.train_step(x.data_ptr(), t.data_ptr(), B, 1e-4)
        torch.cuda.synchronize()
        reps = max(3, args.steps)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(reps):
            net.forward(x.data_ptr(), B, out.data_ptr())
        ev1.record(stream)
        torch.cuda.synchronize()
        fwd_s = ev0.elapsed_time(ev1) / 1e3 / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            net.train_step(x.data_ptr(), t.data_ptr(), B, 1e-4)
        train_s = (time.perf_counter() - t0) / reps  # train_step synchronizes
    res["forward"] = {"ms": fwd_s * 1e3, "tflops": fwd_flops / fwd_s / 1e12, "of_bf16_peak": fwd_flops / fwd_s / 1e12 / peak}
    res["train_step"] = {"ms": train_s * 1e3, "tflops": train_flops / train_s / 1e12,
                         "note": "wall time per synchronous step, host launch overhead included"}
    res["bf16_peak_tflops"] = peak
    print(json.dumps(res), flush=True)


def measured_peaks_tensor():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except (OSError, KeyError, ValueError):
        return 1900.0


def main():
    args = parse()
    if args.study == "cnn":
        run_cnn_study(args)
        return
    if args.study == "learned":
        run_learned_study(args)
        return
    if args.study == "precision":
        run_precision_study(args)
        return
    if args.study == "batched":
        run_batched_study(args)
        return
    if args.study == "rk45":
        run_rk45_study(args)
        return
    if args.study == "wave3d":
        run_wave3d_study(args)
        return
    if args.study == "decomp":
        run_decomp_study(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist = dist_mod
        import torch

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    if args.impl == "reference":
        run_reference(args, rank)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    import numpy as np
    import torch

    import build as gpu_build
    import sbpgpu

    if rank == 0:
        gpu_build.build()
    if dist:
        dist.barrier()
    gpu_build.build()
    torch.cuda.set_device(local)
    n, order = args.grid, args.order
    prec = sbpgpu.FP64 if args.precision == "fp64" else sbpgpu.FP32
    bc = sbpgpu.BC_CHARACTERISTIC if args.bc == "characteristic" else sbpgpu.BC_REFERENCE
    h = 2.0 / (n - 1)
    dt = 0.2 * h
    ctx = sbpgpu.Context(sbpgpu.WAVE_HOM_2D, order, n, n, bc=bc, precision=prec, device=local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    v0 = initial_state(n)
    ctx.set_state(v0)
    ctx.synchronize()

    def sync_all():
        ctx.synchronize()
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        ctx.step_resident(0.0, dt, args.rk_steps)
    sync_all()

    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    sync_all()
    ev0.record(stream)
    for _ in range(args.steps):
        ctx.step_resident(0.0, dt, args.rk_steps)
    ev1.record(stream)
    ctx.synchronize()
    elapsed_ms = ev0.elapsed_time(ev1)
    launches = ctx.launches - launches0
    elapsed_ms = max_over_ranks(elapsed_ms, dist, f"cuda:{local}")
    sync_all()
    clock_info = clocks.stop()

    ms_per_step = elapsed_ms / args.steps
    units_per_step = n * n * 4 * args.rk_steps
    value = world * units_per_step / (ms_per_step * 1e-3)
    es = 8 if args.precision == "fp64" else 4
    scalars_per_pt_step = 16 * 3 if args.precision == "fp64" else 19 * 3
    bytes_per_launch = scalars_per_pt_step * es * n * n / 4.0
    kernel_ms = elapsed_ms / max(launches, 1)
    achieved = bytes_per_launch / (kernel_ms * 1e-3) / 1e9
    peak, peak_src = measured_peaks()
    traffic_pp = profiled_traffic(order, args.precision)
    mid_alg = (5 * 3 * es) * n * n  # algorithmic bytes of one middle-stage launch
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": (traffic_pp * n * n if traffic_pp else None),
                "traffic_note": ("imported, not measured by this run: DRAM bytes of one middle-stage (stage 2/3) "
                                 "launch from the ncu capture summarised in %s (2560^2, scaled by points); "
                                 "that launch's algorithmic bytes: %d" % (profile_summary(order, args.precision),
                                                                          mid_alg)),
                "peak_source": peak_src,
                "algorithmic_bytes_per_launch": bytes_per_launch,
                "kernel": ("wave_fixed_kernel (fused RHS + SAT + RK4 stage, fixed-point stencils)"
                           if args.precision == "fp64" else "wave_stage_kernel (fused RHS + SAT + RK4 stage)"),
                "avg_launch_ms": kernel_ms}
    if args.precision == "fp64":
        try:
            rate = sbpgpu.probe_dfma_rate(local)
            # The fixed-point stages leave only the RK4 update on the FP64 pipe: 2 FMAs per
            # component in stages 1-3, 1 in stage 4 (5.25 per point-stage); the stencils run as
            # int64 on the INT pipe. (The FP64 tap form needed 13.25 / 21.25 / 29.25.)
            dp_ops = 5.25
            roofline["fp64_alu"] = {"dfma_per_s": rate, "dp_instr_per_point_stage": dp_ops,
                                    "bound_point_stage_per_s": rate / dp_ops,
                                    "frac_of_dp_bound": (units_per_step / (ms_per_step * 1e-3)) / (rate / dp_ops)}
        except sbpgpu.SbpError:
            pass

    e2e = None
    if not args.no_e2e:
        host = torch.empty(n * n * 3, dtype=torch.float64, pin_memory=True).numpy()
        times = []
        for k in range(args.warmup + args.steps):
            host[:] = v0
            sync_all()
            t0 = time.perf_counter()
            ctx.rk4_ptr(host.ctypes.data, 0.0, dt, args.rk_steps, sbpgpu.HOST)
            el = time.perf_counter() - t0
            if k >= args.warmup:
                times.append(el)
        el = statistics.median(times)
        el = max_over_ranks(el, dist, f"cuda:{local}")
        e2e = {"value": world * units_per_step / el, "unit": UNIT, "h2d_bytes_per_step": host.nbytes,
               "d2h_bytes_per_step": host.nbytes, "ms_per_step": el * 1e3,
               "call": "sbp_rk4(ctx, 0, dt, steps, host_aos, SBP_HOST)"}

    forms = None
    if rank == 0 and not args.no_forms and args.precision == "fp64":
        forms = measure_forms(peak, local)

    cpu = None
    if rank == 0 and not args.no_cpu:
        rates, kind, threads, sample = cpu_baseline(n, order, args.precision, args.bc, 10.0)
        cpu = {"value": rates[0], "unit": UNIT, "cores": threads, "kind": kind, "sample": sample,
               "port_vs_reference_code": REF_CODE_RATIO}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
                "data": "synthetic (Gaussian pressure pulse)", "config": config_of(args),
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clock_info,
                "gpu_launches": launches, "forms": forms}
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
