#!/usr/bin/env python
"""Benchmark of the batched cloning sampler (one JSON line on rank 0).

Metric: clone lattice updates per second (clone-LUPS) of the whole sampler --
every LB step of every clone plus the cloning step -- on the workload named in
config.workload (default: 4096 clones of a 256x64 channel, FP32 populations
with FP64 drag integral / weights / normaliser, T = 100 LB steps per cloning
interval).  One bench "step" is one cloning interval.

  python bench.py [--steps K] [--warmup W] [--workload c3] [--impl reference]
  torchrun --nproc-per-node N bench.py --gpus N     (independent replicas)

value      device time (CUDA events on the sampler's stream) of K intervals,
           each interval and its cloning step replayed as one CUDA graph
           (--eager: enqueued launch by launch), state resident in HBM; inputs
           (2 x 2.4 GB population buffers) are larger than L2, so no flush is
           needed between intervals.
e2e        the same metric through the C ABI as a driver calls it: the initial
           populations loaded from pinned host memory in the reference's AoS
           FP64 layout, then every interval's drag series, labels, weights and
           R_t delivered to host arrays (clbm_run_sampler_outputs: each
           interval's outputs are copied out while the next interval runs).
roofline   the dominant kernel (the stream-collide step, or the cluster-resident
           interval kernel when the autotuner picks it): algorithmic bytes
           (72 B/LUP FP32, 144 B/LUP FP64: one read and one write of nine
           populations) per step / its mean duration, from CUDA event pairs
           around the step (or interval) launches of one eagerly enqueued
           interval after the timed region; for the cluster-resident kernel an
           HBM-equivalent rate, with its binding resources from its ncu summary.
fp64_same_workload  the same workload in the FP64 mode (the reference's
           arithmetic), for the like-for-like ratio to the CPU baseline.
cpu_baseline the oracle's C port of the reference hot loop on this host's cores.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
PKG = REPO / "cloning-lbm-mpi_gb300"
sys.path.insert(0, str(PKG))
MEASURED_PEAKS = REPO / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0

CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(f"/tmp/clbm_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={CLOCK_FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def hbm_peak():
    try:
        v = json.loads(MEASURED_PEAKS.read_text())["hbm_gbs"]
        return float(v), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel_file: str):
    """dram bytes per launch recorded from an ncu capture in profiles/."""
    p = REPO / "profiles" / kernel_file
    if not p.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch_full_size:\s*([0-9.eE+]+)", p.read_text())
    return float(m.group(1)) if m else None


def ncu_issue_busy(kernel_file: str):
    """issue-slot use of a kernel from its ncu summary in profiles/ (fraction)."""
    p = REPO / "profiles" / kernel_file
    if not p.exists():
        return None
    m = re.search(r"\| issue slots busy \| ([0-9.]+) %", p.read_text())
    return float(m.group(1)) / 100 if m else None


def fp64_same_workload(wl, steps: int = 2):
    """The same workload in FP64 (the reference's arithmetic, bit-identical to
    the oracle): clone-LUPS/s over `steps` intervals after one warm-up,
    CUDA-event timed, state resident."""
    import torch
    import clbm
    s = clbm.Sampler(wl.descs(), clbm.FP64, max_steps=wl.steps, flags=clbm.FLAG_GRAPH)
    for i, r in enumerate(wl.runs):
        s.init_equilibrium(i, r.u0, wl.init_noise, r.seed)
    stream = torch.cuda.ExternalStream(s.stream())
    s.run_sampler(wl.steps, 1)
    s.sync()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    s.run_sampler(wl.steps, steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    s.close()
    return wl.lattice_updates_per_interval * steps / (ms / 1e3)


def dist_setup(args):
    """One process per GPU under torchrun: NCCL for the GPU arm, gloo for the
    reference arm (host cores only; rank 0 alone measures)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        gpu = args.impl != "reference"
        if gpu:
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if gpu else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, x: float) -> float:
    """Maximum of x over the ranks (the slowest rank's time)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(wl, seconds_hint: float = 2.0):
    """The oracle's C port of the reference hot loop (per clone: step, walls,
    square, reset, swap, drag) on all host cores, one clone per thread; the
    sample is ncores clones x S steps of the workload's first lattice."""
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    oracle.build()
    r = wl.runs[0]
    g = oracle.channel_geom(r.width, r.height, r.side, r.xc, r.yc)
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    t, _ = oracle.bench_lbm(g, cores, 20, r.tau, r.beta, cores)
    per_step = t / 20
    steps = max(20, int(seconds_hint / per_step))
    t, _ = oracle.bench_lbm(g, cores, steps, r.tau, r.beta, cores)
    lups = cores * r.nodes * steps
    return {"value": lups / t, "unit": "clone-LUPS/s", "cores": cores, "kind": "port",
            "sample": f"{cores} clones x {steps} LB steps of {r.width}x{r.height} (square {r.side}), "
                      f"FP64, drag every step, {t:.2f} s wall"}


def run_reference(args, wl, world, rank):
    if rank != 0:
        return
    samples = [cpu_sample(wl, 1.0) for _ in range(args.warmup)]  # warm-up, discarded
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s = cpu_sample(wl, 2.0)
        vals.append(s["value"])
    wall = time.perf_counter() - t0
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": "clone-LUPS/s", "value": v, "unit": "clone-LUPS/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * wall / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl.name, "note": "each step is a bounded CPU sample of the workload"},
            "cpu_baseline": {**s, "value": v},
            "e2e": {"value": v, "unit": "clone-LUPS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def precision_study(args, wl):
    """FP32 populations vs the FP64 mode (bit-identical to the oracle) on the
    same GB300 and the same seeds: drag-series error of the first interval,
    SCGF of every run with the FP32 context following the FP64 genealogy
    (precision effect only) and running independently (precision plus the
    genealogy flips it causes), and the speed of both."""
    import torch
    import clbm
    descs = wl.descs()
    ctx = {k: clbm.Sampler(descs, p, max_steps=wl.steps, flags=clbm.FLAG_GRAPH)
           for k, p in (("f64", clbm.FP64), ("f32_locked", clbm.FP32), ("f32_free", clbm.FP32))}
    for s in ctx.values():
        for i, r in enumerate(wl.runs):
            s.init_equilibrium(i, r.u0, wl.init_noise, r.seed)
    n = args.steps
    secs = {}
    drag_err = []
    for t in range(n):
        for k, s in ctx.items():
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.run_interval(wl.steps)
            s.sync()
            secs[k] = secs.get(k, 0.0) + time.perf_counter() - t0
        if t == 0:
            for i in range(len(wl.runs)):
                a, b = ctx["f64"].drag(i), ctx["f32_locked"].drag(i)
                drag_err.append({"max_rel": float(np.abs(b - a).max() / np.abs(a).max()),
                                 "rms_rel": float(np.sqrt(np.mean((b - a) ** 2)) / np.sqrt(np.mean(a ** 2)))})
        for s in ctx.values():
            s.clone_step()
        for i in range(len(wl.runs)):
            ctx["f32_locked"].set_pending_labels(i, ctx["f64"].clone_result(i)["labels"])
    runs = []
    for i, r in enumerate(wl.runs):
        dT = wl.steps * r.dt
        psi = {k: s.scgf(i, dT) for k, s in ctx.items()}
        runs.append({"run": i, "k": r.k, "scgf_fp64": psi["f64"],
                     "scgf_fp32_locked": psi["f32_locked"], "scgf_fp32_free": psi["f32_free"],
                     "scgf_rel_err_locked": abs(psi["f32_locked"] - psi["f64"]) / abs(psi["f64"]),
                     "scgf_rel_err_free": abs(psi["f32_free"] - psi["f64"]) / abs(psi["f64"]),
                     "drag_first_interval": drag_err[i]})
    lups = wl.lattice_updates_per_interval * n
    line = {"study": "precision", "workload": wl.name, "intervals": n, "steps_per_interval": wl.steps,
            "runs": runs, "clone_lups": {k: lups / v for k, v in secs.items()},
            "fp32_over_fp64_speed": secs["f64"] / secs["f32_free"]}
    print(json.dumps(line))


def drag_study(args, wl):
    """Momentum-exchange drag (drag_mode 1) against the reference's stress
    integration (drag_mode 0) on the same workload, seeds and precision:
    per run the first interval's drag series (both estimators on the same
    states), the time-mean drag of every clone over all intervals, the SCGF
    of each sampler, and the cost of each in ms per interval."""
    import torch
    import clbm
    ctx = {}
    for name, mode in (("stress", clbm.DRAG_STRESS), ("momentum", clbm.DRAG_MOMENTUM)):
        descs = wl.descs()
        for d in descs:
            d.drag_mode = mode
        s = clbm.Sampler(descs, wl.precision, max_steps=wl.steps, flags=clbm.FLAG_GRAPH)
        for i, r in enumerate(wl.runs):
            s.init_equilibrium(i, r.u0, wl.init_noise, r.seed)
        if wl.precision == clbm.FP32:
            s.autotune(launches=3)
        ctx[name] = s
    n = args.steps
    secs = {k: 0.0 for k in ctx}
    first = {}
    mean_drag = {k: [np.zeros(r.nclones) for r in wl.runs] for k in ctx}
    for t in range(n):
        for k, s in ctx.items():
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.run_interval(wl.steps)
            s.sync()
            secs[k] += time.perf_counter() - t0
            for i in range(len(wl.runs)):
                dr = s.drag(i)
                mean_drag[k][i] += dr.mean(axis=1) / n
                if t == 0:
                    first[(k, i)] = dr
            s.clone_step()
    runs = []
    for i, r in enumerate(wl.runs):
        a, b = first[("stress", i)], first[("momentum", i)]
        dT = wl.steps * r.dt
        psi = {k: s.scgf(i, dT) for k, s in ctx.items()}
        ma, mb = mean_drag["stress"][i], mean_drag["momentum"][i]
        runs.append({"run": i, "k": r.k,
                     "first_interval": {"mean_stress": float(a.mean()), "mean_momentum": float(b.mean()),
                                        "rms_rel_diff": float(np.sqrt(np.mean((b - a) ** 2) / np.mean(a ** 2)))},
                     "time_mean_drag": {"stress": float(ma.mean()), "momentum": float(mb.mean()),
                                        "rel_diff": float((mb.mean() - ma.mean()) / abs(ma.mean()))},
                     "scgf": psi,
                     "scgf_rel_diff": (psi["momentum"] - psi["stress"]) / abs(psi["stress"])})
    for s in ctx.values():
        s.close()
    line = {"study": "drag", "workload": wl.name, "intervals": n, "steps_per_interval": wl.steps,
            "precision": "fp32" if wl.precision == clbm.FP32 else "fp64", "runs": runs,
            "ms_per_interval": {k: 1e3 * v / n for k, v in secs.items()}}
    print(json.dumps(line))


def adjoint_study(args, wl, directions: int = 32, every: int = 20, eps: float = 1e-6):
    """Gradient of the interval-integrated drag w.r.t. a Gaussian (sigma =
    1e-4) perturbation of all nine populations: FP32 (and FP64) adjoint
    against FP64 central finite differences along random directions."""
    import torch
    import clbm
    r = wl.runs[0]
    descs = wl.descs()
    T = wl.steps
    n = 9 * r.nodes
    rng = np.random.default_rng(r.seed)
    with clbm.Sampler(descs, clbm.FP64, max_steps=T) as f64:
        f64.init_equilibrium(0, r.u0, 1e-3, r.seed)
        base = np.concatenate([f64.dump(0, j) for j in range(r.nclones)])
    S0 = base + rng.normal(0.0, r.noise, base.size)
    out = {}
    grads = {}
    for name, prec in (("fp32", clbm.FP32), ("fp64", clbm.FP64)):
        with clbm.Sampler(descs, prec, max_steps=T) as s:
            s.load_run(0, S0)
            s.drag_fwd(T, every)  # warm-up of both passes (kernel loading)
            s.drag_bwd()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            J = s.drag_fwd(T, every)
            t1 = time.perf_counter()
            s.drag_bwd()
            t2 = time.perf_counter()
            grads[name] = np.concatenate([s.drag_grad(0, j) for j in range(r.nclones)])
            out[name] = {"fwd_s": t1 - t0, "bwd_s": t2 - t1, "J_mean": float(np.mean(J))}
    errs = {"fp32": [], "fp64": []}
    nerrs = {"fp32": [], "fp64": []}  # |ad - fd| / (|g| |d|) per clone and direction
    cos_fd = []                       # |fd| / (|g| |d|): how far the direction is from orthogonal to g
    g64 = grads["fp64"].reshape(r.nclones, n)
    gnorm = np.linalg.norm(g64, axis=1)
    with clbm.Sampler(descs, clbm.FP64, max_steps=T) as f:
        for _ in range(directions):
            d = rng.normal(0.0, 1.0, base.size)
            f.load_run(0, S0 + eps * d)
            jp = f.drag_fwd(T, every)
            f.load_run(0, S0 - eps * d)
            jm = f.drag_fwd(T, every)
            fd = (jp - jm) / (2 * eps)
            dn = np.linalg.norm(d.reshape(r.nclones, n), axis=1)
            cos_fd.extend((np.abs(fd) / (gnorm * dn)).tolist())
            for k in errs:
                ad = (grads[k] * d).reshape(r.nclones, n).sum(axis=1)
                errs[k].extend((np.abs(ad - fd) / np.abs(fd)).tolist())
                nerrs[k].extend((np.abs(ad - fd) / (gnorm * dn)).tolist())
    cos_fd = np.array(cos_fd)
    for k in errs:
        e, ne = np.array(errs[k]), np.array(nerrs[k])
        w = int(np.argmax(e))
        g = grads[k].reshape(r.nclones, n)
        out[k].update({"rel_err_max": float(e.max()), "rel_err_median": float(np.median(e)),
                       "rel_err_p99": float(np.quantile(e, 0.99)),
                       "worst": {"clone": w % r.nclones, "direction": w // r.nclones,
                                 "fd_over_gnorm_dnorm": float(cos_fd[w])},
                       "norm_rel_err_max": float(ne.max()), "norm_rel_err_median": float(np.median(ne)),
                       "grad_rel_l2_vs_fp64_max": float((np.linalg.norm(g - g64, axis=1) / gnorm).max())})
    out["fd_over_gnorm_dnorm"] = {"min": float(cos_fd.min()), "median": float(np.median(cos_fd))}
    lups = r.nclones * r.nodes * T
    line = {"study": "adjoint", "workload": wl.name, "directions": directions, "fd_eps": eps,
            "checkpoint_every": every, "perturbation_sigma": r.noise, "comparisons": len(errs["fp32"]),
            "results": out, "fp32_fwd_bwd_clone_lups": lups / (out["fp32"]["fwd_s"] + out["fp32"]["bwd_s"])}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10, help="timed cloning intervals")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="c3")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--eager", dest="graph", action="store_false",
                    help="enqueue every interval's launches from the host instead of replaying CUDA graphs")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 run of the same workload")
    ap.add_argument("--variant", type=int, default=None,
                    help="use this interval kernel variant instead of autotuning (profiling)")
    ap.add_argument("--band-rows", default=None,
                    help="with --variant: rows per CTA of the cluster-resident kernel, e.g. 24,16,24 (profiling)")
    ap.add_argument("--study", choices=["precision", "adjoint", "drag"], default=None)
    ap.add_argument("--drag", choices=["stress", "momentum"], default="stress",
                    help="drag estimator of the weights (stress: the reference's)")
    args = ap.parse_args()
    from clbm import configs
    wl = configs.WORKLOADS[args.workload]()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, wl, world, rank)
        return
    if args.study == "precision":
        precision_study(args, wl)
        return
    if args.study == "adjoint":
        adjoint_study(args, wl)
        return
    if args.study == "drag":
        drag_study(args, wl)
        return

    import torch
    import clbm
    torch.cuda.set_device(local)
    descs = wl.descs()
    for d in descs:
        d.drag_mode = clbm.DRAG_MOMENTUM if args.drag == "momentum" else clbm.DRAG_STRESS
    s = clbm.Sampler(descs, wl.precision, max_steps=wl.steps,
                     flags=clbm.FLAG_GRAPH if args.graph else 0)
    for i, r in enumerate(wl.runs):
        s.init_equilibrium(i, r.u0, wl.init_noise, r.seed + 1000 * rank)
    stream = torch.cuda.ExternalStream(s.stream())
    s.run_sampler(wl.steps, max(1, args.warmup - 1))
    # autotune the step kernel's launch variant on this workload (state untouched)
    if args.variant is None:
        best, tune_ms = s.autotune(launches=5)
    else:
        s.set_step_variant(args.variant)
        if args.band_rows:
            for i in range(len(wl.runs)):
                s.set_band_rows(i, [int(x) for x in args.band_rows.split(",")])
        best, tune_ms = args.variant, []
    s.run_sampler(wl.steps, 1)
    s.sync()

    # ---- timed region: K intervals, state resident in HBM ----
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.profile(not args.graph)  # event pairs around the step launches (eager replay only)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        rv = s.run_sampler(wl.steps, args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = allmax(world, ev0.elapsed_time(ev1))
    if args.graph:
        # graph replays carry no per-kernel events: time the step launches of
        # one more, eagerly enqueued interval right after the timed region
        s.profile(True)
        s.run_sampler(wl.steps, 1)
    step_ms, nsteps = s.profile_read()
    field_ms, nfield = s.profile_read_fields()
    s.profile(False)
    lups_interval = wl.lattice_updates_per_interval
    value = world * lups_interval * args.steps / (ms / 1e3)
    nodes_total = sum(r.nclones * r.nodes for r in wl.runs)
    bpl = 72 if wl.precision == clbm.FP32 else 144
    step_s = step_ms / 1e3 / max(1, nsteps)
    achieved = bpl * nodes_total / step_s / 1e9
    peak, peak_kind = hbm_peak()
    if wl.precision == clbm.FP32:
        kinds = [clbm.describe_variant(int(v)) for v in s.run_variants()]
        for r, k in enumerate(kinds):  # rows per CTA of each cluster-resident run
            if k["kind"] == "cluster-resident":
                k["band_rows"] = [int(x) for x in s.band_rows(r)]
    else:
        kinds = [{"kind": "streaming", "kernel": "k_step_f64", "variant": 0}] * len(wl.runs)
    n_cluster = sum(k["kind"] == "cluster-resident" for k in kinds)
    any_stream = n_cluster < len(kinds)
    if all(k == kinds[0] for k in kinds):
        vinfo = kinds[0]
    else:  # per-run plan: cluster-resident runs concurrent with the streaming ones
        vinfo = {"kind": "per-run", "kernel": "k_temporal_f32+k_step_f32", "variant": best, "runs": kinds}
    cluster = n_cluster > 0
    # DRAM bytes per launch of the dominant kernel (one step for the streaming
    # kernel, one interval of wl.steps steps for the cluster-resident one)
    traffic = ncu_traffic(f"{vinfo['kernel']}_{args.workload}.md")
    # the interval kernels + drag reduction (2) + cloning step, + the reseed
    # unless every run is cluster-resident with an even interval length (the
    # interval kernels then do the reseed while loading their clones)
    fused = (wl.precision == clbm.FP32 and not any_stream and wl.steps % 2 == 0
             and not any(r.field_steps > 0 for r in wl.runs))
    launches_per_interval = n_cluster + (wl.steps if any_stream else 0) + (3 if fused else 4)
    # the streaming step kernel's own roofline, from the autotuner's timing of
    # its best launch variant on this workload (one launch per step)
    stream_ref = None
    stream_ms = [float(x) for x in tune_ms[:clbm.STREAM_VARIANTS] if x > 0]
    if cluster and stream_ms:
        sms = min(stream_ms)
        sa = bpl * nodes_total / (sms / 1e3) / 1e9
        stream_ref = {"kernel": "k_step_f32", "ms_per_step": sms, "achieved": sa, "frac": sa / peak,
                      "traffic": ncu_traffic(f"k_step_f32_{args.workload}.md")}

    # ---- e2e: initial load from pinned host memory + every interval's outputs on the host ----
    e2e = None
    if not args.no_e2e:
        n = [9 * r.nodes for r in wl.runs]
        host = []
        for i, r in enumerate(wl.runs):
            # the reference's AoS FP64 initial states: one equilibrium field per
            # run replicated over clones (content does not change the cost)
            one = torch.empty(n[i], dtype=torch.float64)
            s.dump(i, 0)  # warm the path
            one.copy_(torch.from_numpy(s.dump(i, 0)))
            h = one.repeat(r.nclones).pin_memory()
            host.append(h)
        # every interval's outputs as the reference writes them per interval
        # (drag series -> data_force.datout, labels, weights; R_t), into host
        # arrays allocated and touched before the timed region
        nct = sum(r.nclones for r in wl.runs)
        out = {"rvalues": np.full((len(wl.runs), args.steps), -1.0),
               "drag": np.full((args.steps, nct, wl.steps), -1.0),
               "labels": np.full((args.steps, nct), -1, np.int32),
               "weights": np.full((args.steps, nct), -1.0)}
        d2h = sum(a.nbytes for a in out.values())
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for i in range(len(wl.runs)):
            clbm.check(clbm.lib().clbm_load_run_aos_f64(s.h, i, host[i].data_ptr()), "load")
        load_s = time.perf_counter() - t0
        h2d = sum(h.numel() * 8 for h in host)
        # the intervals (CUDA graphs unless --eager), each interval's outputs
        # copied to the host while the next one runs
        s.run_sampler_outputs(wl.steps, args.steps, out)
        torch.cuda.synchronize()
        wall = allmax(world, time.perf_counter() - t0)
        assert (out["labels"] >= 0).all() and np.isfinite(out["drag"]).all()
        e2e = {"value": world * lups_interval * args.steps / wall, "unit": "clone-LUPS/s",
               "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps,
               "initial_load": {"ms": 1e3 * load_s, "gb_per_s": h2d / load_s / 1e9},
               "note": "initial AoS FP64 populations from pinned host memory (amortised over the "
                       "steps) + every interval's drag series, labels, weights and R_t delivered to "
                       "host arrays (clbm_run_sampler_outputs: staged while the next interval runs)"}

    s.close()
    fp64 = None
    if wl.precision == clbm.FP32 and not args.no_fp64 and rank == 0:
        fp64 = fp64_same_workload(wl)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_sample(wl)
    if rank != 0:
        return
    clocks = clk.summary()
    line = {
        "metric": "clone-LUPS/s", "value": value, "unit": "clone-LUPS/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if wl.precision == clbm.FP32 else "f64", "data": "synthetic",
        "config": {"workload": wl.name,
                   "runs": [f"{r.nclones}x{r.width}x{r.height} s={r.side} k={r.k:.3f} tau={r.tau}"
                            for r in wl.runs],
                   "steps_per_interval": wl.steps, "parallelism": f"replicas{world}",
                   "drag": args.drag,
                   "step_variant": best,
                   "autotune_ms_per_launch": [round(float(x), 4) for x in tune_ms],
                   "l2": "inputs larger than L2 (two population buffers of "
                         f"{nodes_total * 9 * (4 if wl.precision == clbm.FP32 else 8) / 1e9:.2f} GB)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "kernel": vinfo["kernel"], "variant": vinfo, "bytes_per_lup": bpl,
                     "mean_step_ms": step_ms / max(1, nsteps),
                     **({"note": "cluster-resident interval kernel: each clone's populations stay in "
                                 "the shared memory of one thread-block cluster for all the steps of "
                                 "an interval, so DRAM traffic per launch (traffic, one interval) is "
                                 "a small fraction of the 72 B/LUP a streaming step must move; "
                                 "achieved counts those algorithmic bytes, hence frac > 1 = the gain "
                                 "over the HBM roofline of streaming; it is an HBM-equivalent rate, "
                                 "not HBM utilisation (DRAM is ~1 % busy): the binding resources are "
                                 "under binding; the streaming step kernel's own figures are under "
                                 "streaming_step",
                         "hbm_equivalent": True,
                         "binding": {"resources": "per-step cluster barrier and instruction issue",
                                     "issue_slots_busy": ncu_issue_busy(f"{vinfo['kernel']}_{args.workload}.md"),
                                     "source": f"profiles/{vinfo['kernel']}_{args.workload}.md (ncu)"},
                         "streaming_step": stream_ref} if cluster else {})},
        "fp64_same_workload": None if fp64 is None else {
            "value": fp64, "unit": "clone-LUPS/s",
            "fp32_over_fp64": value / fp64,
            "vs_cpu_baseline": None if cpu is None else fp64 / cpu["value"],
            "note": "the same workload in the FP64 mode (reference arithmetic, bit-identical to the "
                    "oracle), device-timed over 2 intervals: the like-for-like figure against the "
                    "FP64 CPU baseline"},
        **({"field": {"ms_per_interval": field_ms / nfield,
                      "share_of_interval": (field_ms / nfield) / (ms / args.steps),
                      "kernels": "k_field_stage1 + k_field_stage2 (CUDA events around them in the "
                                 "eagerly enqueued intervals)"}} if nfield else {}),
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches_per_interval * args.steps,
        "graph": bool(args.graph),
        "clocks": clocks,
        "rvalues_tail": [float(x) for x in rv[:, -1]],
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
