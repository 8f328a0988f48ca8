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
                   ppc0=16.0, field="turbulent", modes=8, dB=1.0, sample_n=(64, 64, 64),
                   reference_n=(128, 128, 128), precision_n=(64, 64, 64),
                   precision_steps=200, sort_interval=8, bench_steps=8),
    "pair2d": dict(name="2D SR pair plasma 512^2, e-/e+ 16 ppc each, drift +-0.3c, order 1, FP32",
                   dim=2, n=(512, 512, 1), order=1, ppc=16, temp=0.01, drift=0.3, nfilter=0,
                   cfl=0.45, skindepth0=10.0, larmor0=10.0, ppc0=16.0, field="none", modes=0,
                   dB=0.0, sample_n=(128, 128, 1), reference_n=(512, 512, 1),
                   precision_n=(512, 512, 1),
                   precision_steps=100, sort_interval=16, bench_steps=16),
    # magnetized uniform plasma: sigma = (skin depth / Larmor radius)^2 = 10,
    # Maxwell-Juttner theta = 1, uniform B0 along x3
    # two cold beams at +-0.2c (16 ppc each) with weights 1 + 1e-3 cos(k x),
    # k = 2 pi / L; gradient of the final E energy after 400 steps
    "adjoint2d": dict(name="2D two-stream adjoint 256^2, cold beams +-0.2c, 16 ppc each, "
                           "amplitude 1e-3, order 2, FP32, 400 steps, checkpoint every 20",
                      dim=2, n=(256, 256, 1), order=2, ppc=16, beta=0.2, amp=1e-3,
                      skindepth0=10.0, cfl=0.45, steps=400, every=20),
    # Kerr (a = 0.95) quasi-spherical Kerr-Schild grid, r log-spaced in
    # [0.9 r_h, 50 r_g], theta in [0, pi], vertical seed field, e-/e+ at rest
    # injected on the device, 4 pairs per cell on average in r < 6 r_g with
    # weights sqrt(det h) / V0; FP32 with the pusher in FP64 within 3 cells
    # of the horizon (either side)
    "wald2d": dict(name="2D GR Wald problem 1024(r) x 512(theta), a 0.95, vertical field, "
                        "e-/e+ injected on the device, 4 pairs/cell in r < 6, order 2, FP32 with FP64 "
                        "near the horizon",
                   dim=2, n=(1024, 512, 1), order=2, a=0.95, r_max=50.0, ppc=4, r_inject=6.0,
                   cfl=0.5, skindepth0=0.05, larmor0=0.0025, ppc0=2.0, niter=10,
                   sort_interval=0, clear_interval=100, precision_n=(512, 256),
                   precision_steps=200),
    # particle injection and output preparation on the turbulence state (one
    # species pair of 8 ppc each on 256^3): not a step, each kernel timed alone
    "io3d": dict(name="3D injection and output preparation on the 256^3 turbulence state, "
                      "e-/e+ 8 ppc each, FP32", dim=3, n=(256, 256, 256), order=2, ppc=8,
                 temp=0.09, drift=0.0, nfilter=4, cfl=0.45, skindepth0=10.0, larmor0=10.0,
                 ppc0=16.0, field="turbulent", modes=8, dB=1.0, bench_steps=5,
                 sort_interval=8),
    "sweep3d": dict(name="3D SR magnetized uniform plasma 192^3, e-/e+ 32 ppc each, sigma 10, "
                         "theta 1, order 3, FP32 vs FP64", dim=3, n=(192, 192, 192), order=3,
                    ppc=32, temp=1.0, drift=0.0, nfilter=0, cfl=0.45, skindepth0=10.0,
                    larmor0=10.0 / math.sqrt(10.0), ppc0=64.0, field="uniform", modes=0, dB=0.0,
                    sample_n=(24, 24, 24), reference_n=(48, 48, 48),
                    precision_n=(192, 192, 192), precision_steps=1000,
                    sort_interval=4),
}

# algorithmic bytes of the fused push+deposit, FP32: per particle read
# i, dx, u, w and write i, dx, u (prev positions stay in registers); per cell
# the E/B gather (24 B) and the J flush (12 B)
BYTES_PER_PARTICLE = {2: 32 + 28, 3: 40 + 36}
BYTES_PER_CELL = 24 + 12

# DRAM bytes (read + write) per particle of one k_push_deposit_tiled launch,
# from an ncu capture of the same plasma on a 96^3 box (14,155,776 particles:
# 652.1 MB read + 510.3 MB written, the deposit records' lines that leave L2
# before they are read included); traffic grows with the particle count at
# fixed particles per cell, so it scales to the full box by npart
DRAM_BYTES_PER_PARTICLE = {"turb3d": 1162.41e6 / 14155776}

# what binds the dominant kernel beside HBM, from one `ncu --set full` capture
# of the same kernel on a smaller box of the same plasma: instruction issue
# and the shared-memory (l1tex) pipe that carries the fixed-point J atomics
PIPE_LIMITS = {
    "turb3d": {"issue_active_pct": 68.7, "l1tex_shared_atomic_wavefronts_per_particle": 16.6,
               "l1tex_wavefronts_pct": 75.9, "warps_active_pct": 49.7,
               "thread_instructions_per_particle": 2426,
               "fp32_flops_per_particle": 1129,
               "capture": "ncu --set full, one launch on a 96^3 box of the same plasma"},
    "sweep3d": {"issue_active_pct": 55.7, "l1tex_wavefronts_pct": 52.7,
                "l1tex_shared_atomic_wavefronts_per_particle": 50.1, "warps_active_pct": 31.4,
                "capture": "ncu --set full, one launch on a 48^3 box of the same plasma"},
}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_over_ranks(t_ms, units, world, device):
    """Replicas: the job's time is the slowest rank's, its work the sum of
    every rank's units. Returns (max t_ms, total units)."""
    if world <= 1:
        return t_ms, units
    import torch.distributed as dist
    tt = torch.tensor([float(t_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    nn = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(nn)
    return float(tt), float(nn)


def make_setup(w, device, n=None):
    from entity_gb300.inputs import GridSpec, empty_field, make_species, turbulent_field
    n = n or w["n"]
    g = GridSpec(dim=w["dim"], n=n, order=w["order"], real=torch.float32)
    B0 = 1.0 / w["larmor0"]
    if w["field"] == "turbulent":
        EB = turbulent_field(g, B0, w["dB"], w["modes"], seed=2, device=device)
    elif w["field"] == "uniform":
        EB = turbulent_field(g, B0, 0.0, 0, seed=2, device=device)
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


# GB300's nominal HBM3e bandwidth, shown beside the measured denominator
HBM_NOMINAL_GBS = 8000.0


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_sample(w, steps, warmup=1, n=None, sort_interval=0, target_s=10.0):
    """The oracle (the CPU restatement of the reference step, bit-exact with
    the reference's own kernels, OpenMP over all host cores) on a sub-box of
    the workload with the same per-cell content; with sort_interval > 0 it
    sorts by the reference's cell key as often as the GPU arm sorts.
    steps=None times as many steps as fill about target_s seconds, judged
    from the warm-up steps (at least 10, at most 200)."""
    from oracle.oracle import Oracle, lib
    n = n or w["sample_n"]
    g, EB, J, buff, sp = make_setup(w, "cpu", n=n)
    for s in sp:
        s.i_prev = [x.clone() for x in s.i]
        s.dx_prev = [x.clone() for x in s.dx]
    prm = step_prm(g, w, sort_interval)
    o = Oracle(g)
    threads = lib(g.real).orc_max_threads()
    per = 0.0
    for k in range(warmup if steps is not None else max(2, warmup)):
        t0 = time.perf_counter()
        o.step(sp, EB, J, buff, prm, k)
        per = time.perf_counter() - t0
        warmup = k + 1
    if steps is None:
        # the last warm-up step, past the first touch of the arrays
        steps = int(min(200, max(10, round(target_s / max(per, 1e-6)))))
    t0 = time.perf_counter()
    for k in range(steps):
        o.step(sp, EB, J, buff, prm, warmup + k)
    dt = time.perf_counter() - t0
    npart = sum(s.npart for s in sp)
    sort = f"sort every {sort_interval} steps" if sort_interval else "sort off"
    return {"value": npart * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "host_cpus": len(os.sched_getaffinity(0)),
            "sample": (f"{'x'.join(str(v) for v in n[:w['dim']])} cells of the same "
                       f"plasma ({npart} particles), {steps} full steps after {warmup} warm-up, "
                       f"{sort}"), "seconds": dt}


def repo_libraries_mapped():
    """The shared libraries of this repository that the process has mapped."""
    libs = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if len(line.split()) >= 6 else ""
                if path.startswith(ROOT) and ".so" in path:
                    libs.add(os.path.relpath(path, ROOT))
    except OSError:
        return None
    return sorted(libs)


def workload_config(w, args, ncells, npart, world):
    """The config of a bench line, the same for both arms."""
    # i, dx (4 B per axis each), u (3 x 4 B), w (4 B) and the 2-byte tag
    state = npart * (8 * w["dim"] + 18)
    return {"workload": w["name"], "cells": ncells, "particles_per_gpu": npart,
            "sort_interval": args.sort_interval,
            "l2": f"inputs larger than L2 (particle state {state / 1e9:.2f} GB)",
            "parallelism": f"replicas x{world}"}


def precision_twin(w, n, steps, sort_interval, every, timers=False, warm=0, series_out=None):
    """FP32 and FP64 runs of the same plasma from identical initial states
    (the FP32 inputs converted exactly to FP64), each through pic_srpic_step;
    FP64 field energy and particle moments at checkpoints. Returns the error
    of the FP32 run against the FP64 run and both throughputs. With
    series_out, every checkpoint is also appended to that file as a JSON
    line as soon as it is taken."""
    import dataclasses
    from entity_gb300.inputs import empty_field
    from entity_gb300.sim import Context, HostPipe
    g32, EB32, J32, buff32, sp32 = make_setup(w, "cuda", n=n)
    g64 = dataclasses.replace(g32, real=torch.float64)
    EB64 = EB32.double()
    J64, buff64 = empty_field(g64, 3, "cuda"), empty_field(g64, 3, "cuda")
    sp64 = [s.astype(torch.float64) for s in sp32]
    npart = sum(s.npart for s in sp32)
    res = {}
    for tag, (g, EB, J, buff, sp) in (("f64", (g64, EB64, J64, buff64, sp64)),
                                      ("f32", (g32, EB32, J32, buff32, sp32))):
        ctx = Context(g)
        prm = step_prm(g, w, sort_interval)
        series = []

        def probe(k):
            e2, b2 = ctx.field_energy(EB, g.dx)
            m = ctx.particle_moments(sp)
            series.append({"step": k, "field": e2 + b2, "kinetic": m[4], "mgamma": m[0],
                           "p": m[1:4]})
            if series_out:
                with open(series_out, "a") as f:
                    f.write(json.dumps({"precision": tag, **series[-1]}) + "\n")

        probe(0)
        evs = []
        for k in range(steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            if timers and k == warm:
                ctx.timers(True)
            a.record()
            ctx.step(sp, EB, J, buff, prm, k)
            b.record()
            if k >= warm:
                evs.append((a, b))
            if (k + 1) % every == 0 or k + 1 == steps:
                probe(k + 1)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in evs)
        res[tag] = {"series": series, "ms": ms,
                    "value": npart * len(evs) / (ms / 1e3),
                    "phases": ctx.read_timers() if timers else None,
                    "errors": ctx.device_errors()}
        ctx.close()
    s32, s64 = res["f32"]["series"], res["f64"]["series"]
    rel = lambda a, b: abs(a - b) / abs(b) if b != 0 else abs(a - b)
    fe = [rel(a["field"], b["field"]) for a, b in zip(s32, s64)]
    ke = [rel(a["kinetic"], b["kinetic"]) for a, b in zip(s32, s64)]
    pe = [max(abs(x - y) for x, y in zip(a["p"], b["p"])) / b["mgamma"]
          for a, b in zip(s32, s64)]
    tot = lambda s: s["field"] + s["kinetic"]
    return {
        "steps": steps, "cells": list(n[:w["dim"]]), "particles": npart,
        "field_energy_rel_err_final": fe[-1], "field_energy_rel_err_max": max(fe),
        "kinetic_energy_rel_err_final": ke[-1], "kinetic_energy_rel_err_max": max(ke),
        "momentum_err_rel_sum_m_gamma_max": max(pe),
        "energy_drift_f32": rel(tot(s32[-1]), tot(s32[0])),
        "energy_drift_f64": rel(tot(s64[-1]), tot(s64[0])),
        "field_energy_f64_final": s64[-1]["field"], "field_energy_f64_initial": s64[0]["field"],
        "checkpoint_every": every,
        "f32_particle_steps_per_s": res["f32"]["value"],
        "f64_particle_steps_per_s": res["f64"]["value"],
        "device_errors": {"f32": res["f32"]["errors"], "f64": res["f64"]["errors"]},
        "_phases_f32": res["f32"]["phases"], "_ms_f32": res["f32"]["ms"],
    }


def run_reference(args, w):
    """The reference's algorithm on the host cores: the oracle, which is
    bit-exact with the reference's own kernels (tests/test_ref_pin.py). Only
    the oracle is built and loaded here; the product library is not."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import build_oracle
    build_oracle.build()
    n_full = args.cells or w["n"]
    full_cells = math.prod(n_full[:w["dim"]])
    full_npart = 2 * w["ppc"] * full_cells
    base = cpu_sample(w, steps=args.steps, warmup=args.warmup, n=w["reference_n"],
                      sort_interval=args.sort_interval)
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": base["seconds"] / args.steps * 1e3 * full_npart /
                           max(1, 2 * w["ppc"] * math.prod(w["reference_n"][:w["dim"]])),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(w, args, full_cells, full_npart, 1),
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "libraries_mapped": repo_libraries_mapped()}
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
    from entity_gb300.sim import Context, HostPipe
    lib = abi.load()

    g, EB, J, buff, sp = make_setup(w, "cuda", n=args.cells)
    prm = step_prm(g, w, args.sort_interval, sort_tiled=not args.reference_sort_key)
    if args.float_atomics:
        prm.deposit_flags = abi.PIC_PD_FLOAT_ATOMICS
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
    t_max, tot_part = reduce_over_ranks(t_ms, npart, world, "cuda")
    value = tot_part * args.steps / (t_max / 1e3)

    # dominant kernel: the fused push+deposit (both species), timed by events
    pd_ms, pd_n = phases["PushDeposit"]
    bytes_pd = npart * BYTES_PER_PARTICLE[g.dim] + g.ncells() * BYTES_PER_CELL
    achieved = bytes_pd / (pd_ms / pd_n / 1e3) / 1e9
    peak, peak_src = hbm_peak()
    traffic = None
    if args.workload in DRAM_BYTES_PER_PARTICLE and not args.reference_sort_key:
        traffic = DRAM_BYTES_PER_PARTICLE[args.workload] * npart

    # end to end through pic_srpic_step_host with host buffers: every step
    # copies the state in from pinned host memory (EB and each species' i, dx,
    # u, w, tag) and the result out (the same plus J, w only on steps that
    # sort); the pipe overlaps one step's outgoing copies with the next step's
    # incoming ones. The byte counts are means over the timed steps.
    e2e = None
    if not args.no_e2e:
        from entity_gb300.inputs import SpeciesArrays
        pin = lambda t: None if t is None else torch.empty(t.shape, dtype=t.dtype,
                                                           pin_memory=True).copy_(t)
        hsp = [SpeciesArrays([pin(x) for x in s.i], [pin(x) for x in s.dx],
                             [None] * len(s.i_prev), [None] * len(s.dx_prev),
                             [pin(x) for x in s.u], pin(s.w), pin(s.tag), s.mass, s.charge,
                             s.pusher, s.npart, s.index) for s in sp]
        hEB, hJ = pin(EB), pin(J)
        pipe = HostPipe()
        k2 = max(1, args.e2e_steps)
        torch.cuda.synchronize()
        barrier()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        a0.record()
        nin = nout = 0
        for k in range(k2):
            ctx.step_host(pipe, hsp, sp, hEB, EB, hJ, J, buff, prm, args.warmup + args.steps + k)
            bi, bo = pipe.bytes()  # counted as queued: steps that sort copy the weights out too
            nin, nout = nin + bi, nout + bo
        pipe.sync()
        a1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        nin, nout = nin // k2, nout // k2
        pipe.close()
        barrier()
        te, _ = reduce_over_ranks(max(a0.elapsed_time(a1) / 1e3, 1e-9), 0, world, "cuda")
        e2e = {"value": tot_part * k2 / te, "unit": UNIT, "h2d_bytes_per_step": nin,
               "d2h_bytes_per_step": nout, "steps": k2, "wall_s": wall,
               "api": "pic_srpic_step_host"}

    if rank != 0:
        return
    # FP32 against FP64 on a sub-box of the same plasma from identical
    # initial states: the error the FP32 throughput is quoted at
    precision = None
    psteps = w["precision_steps"] if args.precision_steps is None else args.precision_steps
    if psteps > 0:
        precision = precision_twin(w, w["precision_n"], psteps, args.sort_interval, every=50)
        for k in [k for k in precision if k.startswith("_")]:
            del precision[k]
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_sample(w, steps=args.cpu_steps, n=w.get("reference_n"),
                         sort_interval=args.sort_interval)
    # the metric's adjoint/forward ratio, on the two-stream adjoint problem
    adj = None
    if not args.no_adjoint and world == 1:
        wa = WORKLOADS["adjoint2d"]
        _, adj = adjoint_measure(wa, wa["steps"], wa["every"], wa["n"][:2], lib)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(w, args, g.ncells(), npart, world),
        "sort_key": "reference cell key" if args.reference_sort_key else "tile-major",
        "current_sum": ("float atomics" if args.float_atomics
                        else "exact (64-bit fixed point, order-independent)"),
        "ns_per_particle_step": 1e9 / (value / world),
        "phases_ms_per_step": {k: v[0] / max(1, args.steps) for k, v in phases.items()},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "frac_of_nominal_8tbs": achieved / HBM_NOMINAL_GBS,
                     "kernel": "k_push_deposit_tiled (fused push + deposit, both species, "
                               "plus the overflow-list drain)",
                     "bytes_per_launch": bytes_pd, "launch_ms": pd_ms / pd_n,
                     "binding_pipes": PIPE_LIMITS.get(args.workload),
                     "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_src})"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clocks,
        "precision": precision,
        "adjoint": adj,
    }
    print(json.dumps(line), flush=True)


def adjoint_measure(w, nsteps, every, n, lib, h_sweep=(1e-4, 3e-4, 1e-3, 2e-3, 4e-3)):
    """Adjoint/forward cost and gradient checks on the two-stream problem:
    FP32 forward and gradient timed with CUDA events, the FP64 gradient, and
    central differences of both forwards at h = 1e-4 (the stated bar) and
    over a sweep of h for the drift."""
    from entity_gb300 import adjoint as A
    from entity_gb300.sim import Context

    def setup(real):
        g, prm, kappa, k = A.two_stream(n=n, ppc_per_beam=w["ppc"], order=w["order"], real=real,
                                        skindepth0=w["skindepth0"], cfl=w["cfl"])
        return g, prm, kappa, k, Context(g)

    def grads(real, timed=False):
        g, prm, kappa, k, ctx = setup(real)
        beta = torch.tensor(w["beta"], dtype=torch.float64, device="cuda", requires_grad=True)
        amp = torch.tensor(w["amp"], dtype=torch.float64, device="cuda", requires_grad=True)
        sp, U, W, EB0 = A.build(g, kappa, k, beta, amp, w["ppc"], ctx)
        out = {"particles": sum(s.npart for s in sp)}
        if timed:
            # warm-up; the first gradient call allocates the checkpoint slots
            # (timed apart as gradient_first_ms); then the plain forward and
            # the steady-state gradient, both timed
            A.forward_energy(ctx, g, prm, sp, U, W, EB0, min(nsteps, 5))
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            L0 = A.energy(ctx, g, prm, sp, U, W, EB0, nsteps, every)
            torch.autograd.grad(L0, [beta, amp], retain_graph=True)
            e1.record()
            torch.cuda.synchronize()
            out["gradient_first_ms"] = e0.elapsed_time(e1)
            l0 = lib.pic_kernel_launches()
            e0.record()
            out["L_forward"] = A.forward_energy(ctx, g, prm, sp, U, W, EB0, nsteps)
            e1.record()
            torch.cuda.synchronize()
            out["forward_ms"] = e0.elapsed_time(e1)
            out["forward_launches"] = lib.pic_kernel_launches() - l0
            e0.record()
        L = A.energy(ctx, g, prm, sp, U, W, EB0, nsteps, every)
        gb, ga = torch.autograd.grad(L, [beta, amp])
        if timed:
            e1.record()
            torch.cuda.synchronize()
            out["gradient_ms"] = e0.elapsed_time(e1)
        out.update(L=float(L.detach()), dL_dbeta=float(gb), dL_damp=float(ga))
        ctx.close()
        return out

    def fd(real, which, h):
        g, prm, kappa, k, ctx = setup(real)
        vals = []
        for sgn in (1, -1):
            b = w["beta"] + (sgn * h if which == "beta" else 0.0)
            a = w["amp"] + (sgn * h if which == "amp" else 0.0)
            sp, U, W, EB0 = A.build(g, kappa, k, torch.tensor(b, dtype=torch.float64, device="cuda"),
                                    torch.tensor(a, dtype=torch.float64, device="cuda"), w["ppc"],
                                    ctx)
            vals.append(A.forward_energy(ctx, g, prm, sp, U, W, EB0, nsteps))
        ctx.close()
        return (vals[0] - vals[1]) / (2 * h)

    r32 = grads(torch.float32, timed=True)
    r64 = grads(torch.float64)
    rel = lambda a, b: abs(a - b) / abs(b) if b != 0 else abs(a - b)
    # central differences at h = 1e-4 (the stated bar). The in-cell offsets
    # are float at every precision and a cold beam rounds them coherently
    # (~3e-8 cells per step), so the difference quotient of the drift
    # resolves dL/dbeta only to ~1e-3 at h = 1e-4; the sweep over h shows it
    checks = {"h": 1e-4}
    for real, tag, r in ((torch.float32, "f32", r32), (torch.float64, "f64", r64)):
        fb, fa = fd(real, "beta", 1e-4), fd(real, "amp", 1e-4)
        checks[tag] = {"dL_dbeta": r["dL_dbeta"], "fd_dbeta": fb,
                       "rel_err_dbeta": rel(r["dL_dbeta"], fb),
                       "dL_damp": r["dL_damp"], "fd_damp": fa, "rel_err_damp": rel(r["dL_damp"], fa)}
    checks["f64_dbeta_h_sweep"] = [
        {"h": h, "fd_dbeta": v, "rel_err_vs_f64_adjoint": rel(r64["dL_dbeta"], v)}
        for h, v in ((h, fd(torch.float64, "beta", h)) for h in h_sweep)]
    checks["f32_vs_f64"] = {"rel_err_dbeta": rel(r32["dL_dbeta"], r64["dL_dbeta"]),
                            "rel_err_damp": rel(r32["dL_damp"], r64["dL_damp"]),
                            "rel_err_L": rel(r32["L"], r64["L"])}
    return r32, {"ratio_gradient_to_forward": r32["gradient_ms"] / r32["forward_ms"],
                 "forward_ms": r32["forward_ms"], "gradient_ms": r32["gradient_ms"],
                 "gradient_first_ms": r32["gradient_first_ms"], "steps": nsteps,
                 "checkpoint_every": every, "particles": r32["particles"],
                 "L": r32["L"], "L_forward": r32["L_forward"], "checks": checks,
                 "workload": w["name"]}


def run_adjoint(args, w):
    """Adjoint/forward cost and gradient checks on the two-stream problem."""
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from __graft_entry__ import build
    build()
    from entity_gb300 import abi
    lib = abi.load()
    nsteps = args.adjoint_steps or w["steps"]
    every = args.checkpoint_every or w["every"]
    n = (args.cells or w["n"])[:2]
    sampler = ClockSampler(local)
    sampler.start()
    r32, adj = adjoint_measure(w, nsteps, every, n, lib)
    clocks = sampler.stop()
    npart = r32["particles"]
    value = npart * nsteps / (r32["forward_ms"] / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": nsteps,
        "warmup": min(nsteps, 5), "ms_per_step": r32["forward_ms"] / nsteps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": w["name"], "cells": n[0] * n[1], "particles_per_gpu": npart,
                   "checkpoint_every": every, "sort_interval": 0, "parallelism": "replicas x1"},
        "adjoint": adj,
        "gpu_launches": r32["forward_launches"],
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_wald(args, w):
    """GR step throughput on the Wald problem (pic_grpic_step)."""
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from __graft_entry__ import build
    build()
    from entity_gb300 import abi
    from entity_gb300.gr import gr_step_params, horizon_island, wald_setup
    lib = abi.load()
    n = (args.cells or w["n"])[:2]
    g, spec, ctx, fields, species = wald_setup(n=n, a=w["a"], r_max=w["r_max"], order=w["order"],
                                               ppc=w["ppc"], r_inject=w["r_inject"])
    prm = gr_step_params(ctx, cfl=w["cfl"], ppc0=w["ppc0"], skindepth0=w["skindepth0"],
                         larmor0=w["larmor0"], sort_interval=w["sort_interval"],
                         clear_interval=w["clear_interval"])
    island = horizon_island(g, spec)
    npart0 = sum(s.npart for s in species)
    for k in range(args.warmup):
        ctx.grpic_step(species, fields, prm, niter=w["niter"], island=island, step=k,
                       match=ctx.match)
    torch.cuda.synchronize()
    ctx.timers(True)
    sampler = ClockSampler(local)
    sampler.start()
    l0 = lib.pic_kernel_launches()
    ev = []
    steps_particles = 0
    for k in range(args.steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        steps_particles += sum(s.npart for s in species)
        a.record()
        ctx.grpic_step(species, fields, prm, niter=w["niter"], island=island,
                       step=args.warmup + k, match=ctx.match)
        b.record()
        ev.append((a, b))
    torch.cuda.synchronize()
    clocks = sampler.stop()
    launches = lib.pic_kernel_launches() - l0
    ms = sum(a.elapsed_time(b) for a, b in ev)
    phases = ctx.read_timers()
    errs = ctx.device_errors()
    value = steps_particles / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w["name"], "cells": n[0] * n[1], "particles_initial": npart0,
                   "particles_final": sum(s.npart for s in species), "dt": prm.dt,
                   "fp64_island_cells": list(island), "match_ds": ctx.match[0],
                   "parallelism": "replicas x1"},
        "ns_per_particle_step": 1e9 / value,
        "phases_ms_per_step": {k: v[0] / max(1, args.steps) for k, v in phases.items()},
        "device_errors": errs,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    psteps = w["precision_steps"] if args.precision_steps is None else args.precision_steps
    if psteps > 0:
        line["precision"] = wald_precision(w, w["precision_n"], psteps)
    print(json.dumps(line), flush=True)


def wald_precision(w, n, steps):
    """The FP32 step (with and without the FP64 island) against the FP64
    step from the same seeded Wald set-up: relative L2 error of D and B,
    and the particle state error of particles alive in all three runs
    (dead particles are not removed, so indices stay aligned)."""
    from entity_gb300.gr import gr_step_params, horizon_island, wald_setup
    runs = {}
    # every run starts from the FP32 injection (a double injection draws
    # 53-bit uniforms, i.e. other positions)
    _, _, _, _, species32 = wald_setup(n=n, a=w["a"], r_max=w["r_max"], order=w["order"],
                                       ppc=w["ppc"], r_inject=w["r_inject"], real=torch.float32)
    for tag, real, isl in (("f64", torch.float64, True), ("f32_island", torch.float32, True),
                           ("f32_no_island", torch.float32, False)):
        g, spec, ctx, fields, _ = wald_setup(n=n, a=w["a"], r_max=w["r_max"], order=w["order"],
                                             ppc=w["ppc"], r_inject=w["r_inject"], real=real)
        species = [s.astype(real) for s in species32]
        prm = gr_step_params(ctx, cfl=w["cfl"], ppc0=w["ppc0"], skindepth0=w["skindepth0"],
                             larmor0=w["larmor0"], sort_interval=0, clear_interval=0)
        island = horizon_island(g, spec) if isl else (0, 0)
        for k in range(steps):
            ctx.grpic_step(species, fields, prm, niter=w["niter"], island=island, step=k,
                           match=ctx.match)
        torch.cuda.synchronize()
        ng = g.ng
        em = fields[0][:, 0, ng:ng + n[1], ng:ng + n[0]].double()
        X = [torch.stack([s.i[d].double() + s.dx[d].double() for d in range(2)]) for s in species]
        U = [torch.stack([u.double() for u in s.u]) for s in species]
        alive = [s.tag == 1 for s in species]
        runs[tag] = (em, X, U, alive, island)
    ref = runs["f64"]
    out = {"steps": steps, "cells": list(n), "fp64_island_cells": list(runs["f32_island"][4])}
    for tag in ("f32_island", "f32_no_island"):
        em, X, U, alive, _ = runs[tag]
        both = [a & b for a, b in zip(alive, ref[3])]
        dx = max(float((x - xr)[:, m].abs().max()) if m.any() else 0.0
                 for x, xr, m in zip(X, ref[1], both))
        du = max(float(((u - ur)[:, m]).norm() / (ur[:, m].norm() + 1e-300)) if m.any() else 0.0
                 for u, ur, m in zip(U, ref[2], both))
        out[tag] = {
            "D_rel_l2": float((em[:3] - ref[0][:3]).norm() / ref[0][:3].norm()),
            "B_rel_l2": float((em[3:] - ref[0][3:]).norm() / ref[0][3:].norm()),
            "x_max_abs_cells": dx, "u_rel_l2": du,
            "alive_mismatch": int(sum(int((a != b).sum()) for a, b in zip(alive, ref[3]))),
        }
    return out


def run_sweep(args, w):
    """The FP32 vs FP64 precision sweep as its own line: both precisions run
    the full workload for warmup + steps steps from identical initial states;
    `value` is the FP32 throughput over the timed steps."""
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from __graft_entry__ import build
    build()
    from entity_gb300 import abi
    lib = abi.load()
    n = args.cells or w["n"]
    total = args.warmup + args.steps
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = lib.pic_kernel_launches()
    pr = precision_twin(w, n, total, args.sort_interval, every=args.checkpoint_every or 50,
                        timers=True, warm=args.warmup, series_out=args.series_out)
    launches = lib.pic_kernel_launches() - launches0
    clocks = sampler.stop()
    phases = pr.pop("_phases_f32")
    ms = pr.pop("_ms_f32")
    value = pr["f32_particle_steps_per_s"]
    npart = pr["particles"]
    ncells = math.prod(n[:w["dim"]])
    pd_ms, pd_n = phases["PushDeposit"]
    bytes_pd = npart * BYTES_PER_PARTICLE[w["dim"]] + ncells * BYTES_PER_CELL
    achieved = bytes_pd / (pd_ms / pd_n / 1e3) / 1e9
    peak, peak_src = hbm_peak()
    cpu = None if args.no_cpu_baseline else cpu_sample(
        w, steps=args.cpu_steps, n=w.get("reference_n"), sort_interval=args.sort_interval)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w["name"], "cells": ncells, "particles_per_gpu": npart,
                   "sort_interval": args.sort_interval, "sort_key": "tile-major",
                   "l2": "inputs larger than L2", "parallelism": "replicas x1"},
        "ns_per_particle_step": 1e9 / value,
        "phases_ms_per_step": {k: v[0] / max(1, args.steps) for k, v in phases.items()},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "frac_of_nominal_8tbs": achieved / HBM_NOMINAL_GBS,
                     "kernel": "k_push_deposit_tiled (FP32, both species)",
                     "bytes_per_launch": bytes_pd, "launch_ms": pd_ms / pd_n,
                     "binding_pipes": PIPE_LIMITS.get("sweep3d"),
                     "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_src})"},
        "precision": pr,
        "cpu_baseline": cpu,
        "e2e": None,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_io(args, w):
    """Injection and output preparation, each timed alone with CUDA events
    on a resident state larger than L2; algorithmic bytes per call against
    the measured HBM peak."""
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from __graft_entry__ import build
    build()
    from entity_gb300 import abi
    from entity_gb300.inputs import empty_field, empty_species, inject_params
    from entity_gb300.sim import Context
    lib = abi.load()
    g, EB, J, buff, sp = make_setup(w, "cuda", n=args.cells)
    prm = step_prm(g, w, w["sort_interval"], sort_tiled=True)
    ctx = Context(g)
    ctx.step(sp, EB, J, buff, prm, 0)   # fills the ghosts and tile-sorts
    torch.cuda.synchronize()
    npart = sum(s.npart for s in sp)
    ncells = g.ncells()
    rb = 4
    peak, peak_src = hbm_peak()
    reps = max(3, args.steps)
    launches0 = lib.pic_kernel_launches()
    sampler = ClockSampler(local)
    sampler.start()

    def timed(fn, nbytes, per):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / reps
        gbs = nbytes / (ms / 1e3) / 1e9
        return {"ms": ms, "GB/s": gbs, "frac": gbs / peak, "bytes_per_call": nbytes,
                "algorithmic_bytes": per}

    out = {}
    # injection: both species of a pair appended to empty species, i, dx, u,
    # w, tag written per particle (the prev arrays are not written)
    cap = sp[0].npart
    e1 = empty_species(g, cap, charge=-1.0, index=1)
    e2 = empty_species(g, cap, charge=1.0, index=2)
    ip = inject_params(1.0, 2.0 * w["ppc"], [(0, g.n[d]) for d in range(3)],
                       (w["temp"], w["temp"]), seed=9)
    per_inj = 3 * 4 + 3 * 4 + 4 * rb + 2

    def inject():
        e1.npart = e2.npart = 0
        ctx.inject_uniform_maxwellians(e1, e2, ip)
    inject()
    torch.cuda.synchronize()
    out["pic_inject_uniform_maxwellians"] = timed(inject, (e1.npart + e2.npart) * per_inj,
                                                  f"{per_inj} B written per particle")
    out["pic_inject_uniform_maxwellians"]["particles_per_s"] = (
        (e1.npart + e2.npart) / (out["pic_inject_uniform_maxwellians"]["ms"] / 1e3))
    del e1, e2
    torch.cuda.empty_cache()
    # moments: N at order 2 (27 cells per particle), T^{0i} at order 0
    bckp = empty_field(g, 6, "cuda")

    def mom(mid, order, c1=0, c2=0):
        p = abi.PicMomentParams()
        p.id, p.c1, p.c2, p.order, p.smoothing = mid, c1, c2, order, abi.PIC_SMOOTH_SPLINE
        p.use_weights, p.inv_n0, p.dx = 1, 1.0 / w["ppc0"], g.dx
        return p
    pn, pt = mom(abi.PIC_MOM_N, 2), mom(abi.PIC_MOM_T, 0, 0, 1)
    per_n = 3 * 4 + 3 * 4 + rb + 2
    out["pic_output_moment N order 2"] = timed(
        lambda: ctx.output_moment(sp, pn, bckp, 0), npart * per_n + ncells * 4,
        f"{per_n} B read per particle + 4 B per cell")
    per_t = per_n + 3 * rb
    out["pic_output_moment T01 order 0"] = timed(
        lambda: ctx.output_moment(sp, pt, bckp, 1), npart * per_t + ncells * 4,
        f"{per_t} B read per particle + 4 B per cell")
    out["pic_sync_moments"] = timed(lambda: ctx.sync_moments(bckp, 0, 2), 0, "ghost slabs only")
    # fields at cell centres in the tetrad basis, no downsampling
    fo = torch.empty((3,) + tuple(reversed(g.n)), dtype=g.real, device="cuda")
    flags = abi.PIC_OUT_INTERP_EDGES | abi.PIC_OUT_TO_HAT
    out["pic_output_field E"] = timed(
        lambda: ctx.output_field(EB, 1, 0, 3, flags, g.dx, (1, 1, 1), fo), ncells * 24,
        "12 B read + 12 B written per cell")
    # every particle as a record in physical units (stride 1)
    n0 = sp[0].npart
    xs = [torch.empty(n0, dtype=g.real, device="cuda") for _ in range(3)]
    us = [torch.empty(n0, dtype=g.real, device="cuda") for _ in range(3)]
    ws = torch.empty(n0, dtype=g.real, device="cuda")
    per_p = (3 * 4 + 3 * 4 + 4 * rb) + 7 * rb
    out["pic_output_particles stride 1"] = timed(
        lambda: ctx.output_particles(sp[0], 1, g.dx, (0.0, 0.0, 0.0), xs, us, ws), n0 * per_p,
        f"{per_p} B per particle (i, dx, u, w read; x, u, w written)")
    clocks = sampler.stop()
    launches = lib.pic_kernel_launches() - launches0
    top = out["pic_output_moment N order 2"]
    line = {
        "metric": "output-preparation throughput (particle moments, fields, particle "
                  "records) and device injection on 1 GB300",
        "value": npart / (top["ms"] / 1e3), "unit": "particles/s (N moment, order 2)",
        "n_gpus": 1, "steps": reps, "warmup": args.warmup, "ms_per_step": top["ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": w["name"], "cells": ncells,
                                        "particles_per_gpu": npart,
                                        "l2": "inputs larger than L2"},
        "kernels": out,
        "roofline": {"bound": "hbm", "achieved": top["GB/s"], "peak": peak, "unit": "GB/s",
                     "frac": top["frac"], "traffic": None,
                     "kernel": "k_output_moment (N, order 2, global atomics)",
                     "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_src})"},
        "cpu_baseline": None, "e2e": None, "gpu_launches": launches, "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: the workload's, a multiple of its sort "
                         "interval so that the window holds its share of sorts)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="turb3d", choices=sorted(WORKLOADS))
    ap.add_argument("--sort-interval", type=int, default=None,
                    help="steps between tile-major sorts (default: the workload's)")
    ap.add_argument("--reference-sort-key", action="store_true",
                    help="sort by the reference's i1-major cell key (untiled push/deposit)")
    ap.add_argument("--cells", type=int, nargs="+", default=None,
                    help="override the grid (smaller cases for profiling)")
    ap.add_argument("--e2e-steps", type=int, default=16)
    ap.add_argument("--cpu-steps", type=int, default=None,
                    help="timed oracle steps of cpu_baseline (default: about 10 s of work, at least 10 steps)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the two-stream adjoint block of the default line")
    ap.add_argument("--precision-steps", type=int, default=None,
                    help="steps of the FP32-vs-FP64 twin on the sub-box (0 = skip)")
    ap.add_argument("--checkpoint-every", type=int, default=None,
                    help="steps between FP64 diagnostics (sweep3d, default 50) or between "
                         "adjoint checkpoints (adjoint2d, default 20)")
    ap.add_argument("--float-atomics", action="store_true",
                    help="deposit with float atomics instead of the exact accumulation")
    ap.add_argument("--series-out", default=None,
                    help="sweep3d: append each FP32/FP64 checkpoint to this file as it is taken")
    ap.add_argument("--adjoint-steps", type=int, default=None,
                    help="forward steps of the adjoint workload (default 400)")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.sort_interval is None:
        args.sort_interval = w.get("sort_interval", 4)
    if args.steps is None:
        args.steps = w.get("bench_steps", 10)
    if args.cells is not None:
        c = list(args.cells) + [1] * (3 - len(args.cells))
        args.cells = tuple(c)
    if args.impl == "reference":
        run_reference(args, w)
    elif args.workload == "sweep3d":
        run_sweep(args, w)
    elif args.workload == "adjoint2d":
        run_adjoint(args, w)
    elif args.workload == "wald2d":
        run_wald(args, w)
    elif args.workload == "io3d":
        run_io(args, w)
    else:
        run_ours(args, w)


if __name__ == "__main__":
    main()
