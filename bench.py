#!/usr/bin/env python
"""Benchmark of the SR particle-in-cell step on GB300.

Workload (default, `turb3d`): 3D Cartesian decaying turbulence, 256^3 cells,
periodic, e-/e+ with 8 particles per cell each (268,435,456 particles),
B = B0 z + 8 random-phase Fourier modes (|k| = 2 pi/L * 1..2, dB/B0 = 1),
Maxwell-Juttner temperature 0.09 (u_th = 0.3 c), shape order 2, 4 filter
passes, CFL 0.45, FP32. Inputs are seeded synthetic data made on the device.

One step = SRPICEngine::step_forward through the library's host engine
(pic_srpic_step): Faraday/2, fused push+deposit of both species, J fold,
4 filter passes, Faraday/2, Ampere + J->E, and a cell sort of both species
every `--sort-interval` steps.

Prints one JSON line (see the keys below). `--impl reference` times the CPU
restatement of the reference's algorithm (the oracle; the reference itself
cannot be built here) on the host cores on a bounded sample of the same
workload.
"""
import argparse
import csv
import io
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import torch  # noqa: E402

METRIC = ("particle-steps/s on 1 GB300: FP32 vs FP64 path at stated error; "
          "adjoint/fwd ratio")
UNIT = "particle-steps/s"

WORKLOADS = {
    "turb3d": dict(name="3D SR decaying turbulence 256^3, e-/e+ 8 ppc each, order 2, "
                        "4 filter passes, FP32", dim=3, n=(256, 256, 256), order=2, ppc=8,
                   temp=0.09, drift=0.0, nfilter=4, cfl=0.45, skindepth0=10.0, larmor0=10.0,
                   ppc0=16.0, modes=8, dB=1.0, sample_n=(64, 64, 64)),
    "pair2d": dict(name="2D SR pair plasma 512^2, e-/e+ 16 ppc each, drift +-0.3c, order 1, FP32",
                   dim=2, n=(512, 512, 1), order=1, ppc=16, temp=0.01, drift=0.3, nfilter=0,
                   cfl=0.45, skindepth0=10.0, larmor0=10.0, ppc0=16.0, modes=0, dB=0.0,
                   sample_n=(128, 128, 1)),
}

# algorithmic bytes of the fused push+deposit, FP32: per particle read
# i, dx, u, w and write i, dx, u (prev positions stay in registers); per cell
# the E/B gather (24 B) and the J flush (12 B)
BYTES_PER_PARTICLE = {2: 32 + 28, 3: 40 + 36}
BYTES_PER_CELL = 24 + 12


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_setup(w, device, n=None):
    from entity_gb300.inputs import GridSpec, empty_field, make_species, turbulent_field
    from entity_gb300.sim import step_params
    n = n or w["n"]
    g = GridSpec(dim=w["dim"], n=n, order=w["order"], real=torch.float32)
    B0 = 1.0 / w["larmor0"]
    if w["modes"] > 0:
        EB = turbulent_field(g, B0, w["dB"], w["modes"], seed=2, device=device)
    else:
        EB = empty_field(g, 6, device)
    J = empty_field(g, 3, device)
    buff = empty_field(g, 3, device)
    sp = [make_species(g, w["ppc"], w["temp"], w["drift"], 11, charge=-1.0, index=1,
                       device=device, with_prev=False),
          make_species(g, w["ppc"], w["temp"], -w["drift"], 12, charge=1.0, index=2,
                       device=device, with_prev=False)]
    return g, EB, J, buff, sp


def step_prm(g, w, sort_interval, sort_tiled=True):
    from entity_gb300.sim import step_params
    return step_params(g, cfl=w["cfl"], ppc0=w["ppc0"], skindepth0=w["skindepth0"],
                       larmor0=w["larmor0"], nfilter=w["nfilter"], sort_interval=sort_interval,
                       write_prev=False, sort_tiled=sort_tiled)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.f.read())) if len(r) >= 9]
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        smax = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows)}


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_sample(w, steps, warmup=1):
    """The oracle (CPU restatement of the reference step, OpenMP over all host
    cores) on a sub-box of the workload with the same per-cell content."""
    from oracle.oracle import Oracle, lib
    g, EB, J, buff, sp = make_setup(w, "cpu", n=w["sample_n"])
    for s in sp:
        s.i_prev = [x.clone() for x in s.i]
        s.dx_prev = [x.clone() for x in s.dx]
    prm = step_prm(g, w, 0)
    o = Oracle(g)
    threads = lib(g.real).orc_max_threads()
    for k in range(warmup):
        o.step(sp, EB, J, buff, prm, k)
    t0 = time.perf_counter()
    for k in range(steps):
        o.step(sp, EB, J, buff, prm, warmup + k)
    dt = time.perf_counter() - t0
    npart = sum(s.npart for s in sp)
    return {"value": npart * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"{'x'.join(str(v) for v in w['sample_n'][:w['dim']])} cells of the same "
                       f"plasma ({npart} particles), {steps} full steps after {warmup} warm-up, "
                       f"sort off"), "seconds": dt}


def run_reference(args, w):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from __graft_entry__ import build
    build()
    base = cpu_sample(w, steps=args.steps, warmup=args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": base["seconds"] / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["name"], "sample": base["sample"]},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, w):
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from __graft_entry__ import build
    build()
    from entity_gb300 import abi
    from entity_gb300.sim import Context
    lib = abi.load()

    g, EB, J, buff, sp = make_setup(w, "cuda", n=args.cells)
    prm = step_prm(g, w, args.sort_interval, sort_tiled=not args.reference_sort_key)
    ctx = Context(g)
    npart = sum(s.npart for s in sp)
    torch.cuda.synchronize()

    # warm-up (step 0 also fills the field ghosts and sorts)
    for k in range(args.warmup):
        ctx.step(sp, EB, J, buff, prm, k)
    torch.cuda.synchronize()
    ctx.timers(True)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    sampler = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    launches0 = lib.pic_kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for k in range(args.steps):
        ctx.step(sp, EB, J, buff, prm, args.warmup + k)
    ev1.record()
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    launches = lib.pic_kernel_launches() - launches0
    t_ms = ev0.elapsed_time(ev1)
    phases = ctx.read_timers()
    ctx.timers(False)
    t_max = t_ms
    tot_part = npart
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt)
        nn = torch.tensor([float(npart)], device="cuda")
        dist.all_reduce(nn)
        tot_part = float(nn)
    value = tot_part * args.steps / (t_max / 1e3)

    # dominant kernel: the fused push+deposit (both species), timed by events
    pd_ms, pd_n = phases["PushDeposit"]
    bytes_pd = npart * BYTES_PER_PARTICLE[g.dim] + g.ncells() * BYTES_PER_CELL
    achieved = bytes_pd / (pd_ms / pd_n / 1e3) / 1e9
    peak, peak_src = hbm_peak()

    # end to end through pic_srpic_step with host buffers: every step copies
    # the full particle and field state from pinned host memory and back
    e2e = None
    if not args.no_e2e:
        tensors = [EB, J, buff]
        for s in sp:
            tensors += [*s.i[:g.dim], *s.dx[:g.dim], *s.u, s.w, s.tag]
        host = [torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in tensors]
        for h, t in zip(host, tensors):
            h.copy_(t)
        nbytes = sum(t.numel() * t.element_size() for t in tensors)
        k2 = max(1, min(args.steps, args.e2e_steps))
        torch.cuda.synchronize()
        barrier()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        a0.record()
        for k in range(k2):
            for h, t in zip(host, tensors):
                t.copy_(h, non_blocking=True)
            ctx.step(sp, EB, J, buff, prm, args.warmup + args.steps + k)
            for h, t in zip(host, tensors):
                h.copy_(t, non_blocking=True)
        a1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        barrier()
        te = max(a0.elapsed_time(a1) / 1e3, 1e-9)
        e2e = {"value": tot_part * k2 / te, "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes, "steps": k2, "wall_s": wall}

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_sample(w, steps=args.cpu_steps)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w["name"], "cells": g.ncells(), "particles_per_gpu": npart,
                   "sort_interval": args.sort_interval,
                   "sort_key": "reference cell key" if args.reference_sort_key else "tile-major",
                   "l2": "inputs larger than L2 (particle state > 10 GB per step)",
                   "parallelism": f"replicas x{world}"},
        "ns_per_particle_step": 1e9 / (value / world),
        "phases_ms_per_step": {k: v[0] / max(1, args.steps) for k, v in phases.items()},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "k_push_deposit (fused push + deposit, both species, J zero)",
                     "bytes_per_launch": bytes_pd, "launch_ms": pd_ms / pd_n,
                     "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_src})"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="turb3d", choices=sorted(WORKLOADS))
    ap.add_argument("--sort-interval", type=int, default=4)
    ap.add_argument("--reference-sort-key", action="store_true",
                    help="sort by the reference's i1-major cell key (untiled push/deposit)")
    ap.add_argument("--cells", type=int, nargs="+", default=None,
                    help="override the grid (smaller cases for profiling)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.cells is not None:
        c = list(args.cells) + [1] * (3 - len(args.cells))
        args.cells = tuple(c)
    if args.impl == "reference":
        run_reference(args, w)
    else:
        run_ours(args, w)


if __name__ == "__main__":
    main()
