#!/usr/bin/env python
"""Benchmark of the coupled MD/MPC cycle on GB300.

A "step" is one cycle: 10 velocity-Verlet MD substeps of every monomer plus
one SRD collision of every solvent particle (stream, Lees-Edwards wrap,
random-shift binning, thermostat + rotation), for every replica.

Headline metric: MPC particle-updates/s = sum over replicas of
(solvent + monomers) x cycles / s. Default workload: batched_256 (256 uneven
boxes, 65.8M solvent particles, FP32 state, one CUDA graph per cycle).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
  python bench.py --impl reference ...   # the CPU implementation on the host cores

Timing: W untimed warm-up cycles, then K cycles bracketed by CUDA events on
the library's own stream (barrier + synchronize on both sides), max over
ranks. The state (>2 GB for batched_256) is far larger than the 129 MB L2.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import csv
import io
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "MPC particle-updates/s"
UNIT = "particle-updates/s"
PHASE_LAUNCHES = 10  # kernels per cycle: md, begin, mono_prep, fluid_bin, 3x scan, perm, collide, end
PMD_LAUNCHES = 2     # kernels per MD substep of a periodic box (nlist, forces), plus 2 per cycle
REF_MAX_STEPS = 20   # timed cycles of the reference arm (each ~0.6 s for batched_256 on 16 cores)


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched_256")
    ap.add_argument("--no-extras", action="store_true", help="skip FP64 ratio, e2e, CPU baseline")
    ap.add_argument("--replicas", type=int, default=0,
                    help="batched_256 only: use the first N replicas (small profiling case)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"],
                    help="state precision of the timed path (fp64: the plain FP64 path the "
                         "drop-in uses, batched like the FP32 one)")
    return ap.parse_args()


# ----------------------------------------------------------------- helpers

def dist_setup(args):
    """One process per GPU under torchrun (RANK, LOCAL_RANK, WORLD_SIZE, MASTER_*).
    NCCL on GPU machines; gloo where no GPU is visible (host-side tests) or when
    SMPC_DIST_BACKEND names it."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = os.environ.get("SMPC_DIST_BACKEND") or (
            "nccl" if torch.cuda.is_available() else "gloo")
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units, steps, world, ms_max):
    """Whole-job throughput: every rank processes `units` per step (replicas
    only, weak scaling), timed by the slowest rank."""
    return units * steps * world / (ms_max / 1e3)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50", "-i", str(self.gpu)], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def rows_written(self):
        if self.proc is None:
            return 1
        try:
            with open(self.tmp.name) as f:
                return sum(1 for line in f if line.count(",") >= 8)
        except OSError:
            return 0

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        self.tmp.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.tmp.read())) if len(r) >= 9]
        os.unlink(self.tmp.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[5 + k]
                          and "Not" not in r[5 + k]})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows), "period_ms": 50,
                "window": "timed region plus untimed cycles of the same work just before "
                          "and after it (the sampler's first row arrives under load)"}


# ------------------------------------------------------------ CPU baseline

def cpu_systems(workload, n_threads, max_replicas=None, all_replicas=False):
    """The oracle (C restatement of the reference, FP64) set up on the host for
    the workload: every replica (``all_replicas``) or a sample of one replica
    per thread. Returns ([(system, particles)], description)."""
    from oracle import oracle as orc
    from starpolymersmd_gb300 import system, workloads as W

    if workload in W.SOLUTIONS:
        pick = [W.SOLUTION_SPECS[workload]()]
    elif workload == "batched_256":
        specs = system.batched_replica_table(256)
        pick = specs if all_replicas else specs[:: max(1, len(specs) // n_threads)][:n_threads]
    elif workload in ("single_star_50", "single_star_50_periodic"):
        # the reference's one-star model (the periodic variant's MD is the
        # same physics while the star has no self-image, see star_extent)
        pick = [system.ReplicaSpec(L=50, arms=10, n_arm=40, solvophobic_fraction=0.5,
                                   shear=0.05, seed=1)]
    else:
        pick = [system.ReplicaSpec(L=20, arms=6, n_arm=20, solvophobic_fraction=0.5,
                                   shear=0.05, seed=1)]
    if max_replicas:
        pick = pick[:max_replicas]

    def make(spec):
        rng = np.random.default_rng(2000 + spec.seed)
        st = W.make_solution(spec) if workload in W.SOLUTIONS else W.compact_star(spec)
        mol_start = st.mol_start if workload in W.SOLUTIONS else [0, st.n]
        mass = st.mass if workload in W.SOLUTIONS else np.full(st.n, st.mass)
        L = spec.L
        fpos, fvel = system.uniform_fluid((L, L, L), spec.n_c, spec.kT, rng)
        o = orc.OracleSystem((L, L, L), spec.kT, spec.shear, W.N_SUB, len(fpos), st.n,
                             mol_start=mol_start, lambda_=1.0, md_dt=W.MD_DT,
                             r_cut=W.R_CUT_LJ, r_verlet=W.R_CUT_LJ + W.SKIN,
                             potential=orc.POT_LJ126, delrx_dt_scale=1.0 / W.N_SUB, mono_wrap=1)
        mvel = st.vel
        if workload in W.SOLUTIONS:  # the steady shear flow, as the GPU workload starts
            fvel[:, 0] += spec.shear * fpos[:, 1]
            mvel = st.vel.copy()
            mvel[:, 0] += spec.shear * st.pos[:, 1]
        o.set_fluid(fpos, fvel)
        n_f = len(fpos)
        del fpos, fvel
        o.set_monomers(st.pos, mvel, np.zeros_like(st.pos), mass, st.amphi, st.anchor)
        o.set_bonds(st.bond_src, st.bond_dst)
        if workload in W.SOLUTIONS:
            o.set_periodic_md(W.H)
        o.init_md()
        o.set_philox(spec.seed, 0)
        return [o, n_f + st.n, 0]

    systems = [make(s) for s in pick]
    desc = (f"oracle C restatement (FP64), {len(systems)} replica(s) of {workload} "
            f"({', '.join(f'L={s.L}' for s in pick[:6])}{'...' if len(pick) > 6 else ''}), "
            f"replicas shared out over {n_threads} thread(s)")
    return systems, desc


def cpu_run(systems, n_threads, cycles):
    """``cycles`` cycles of every system, the systems shared out over a pool of
    host threads (the C oracle releases the GIL). Returns (units, seconds)."""
    from starpolymersmd_gb300 import workloads as W

    def run(item):
        o, units, done = item
        # t = done*N_SUB + 1 ...: collisions every N_SUB calls, continuing the run
        o.run(done * W.N_SUB + 1, W.N_SUB * cycles, W.H, True)
        item[2] = done + cycles
        return units * cycles

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=n_threads) as ex:
        units = sum(ex.map(run, systems))
    return units, time.perf_counter() - t0


def cpu_sample(workload, n_threads, cycles, max_replicas=None):
    """The oracle on host cores: one replica per thread, ``cycles`` cycles
    each. Returns (units/s, description, units, seconds)."""
    systems, desc = cpu_systems(workload, n_threads, max_replicas)
    units, dt = cpu_run(systems, n_threads, cycles)
    return units / dt, desc + f", {cycles} cycle(s) each", units, dt


def cpu_cycles_for(workload, n_threads):
    # about 10-30 s of CPU work in total
    return {"batched_256": 20, "single_star_50": 5, "single_star_20": 40, "semidilute_100": 3,
            "large_box_200": 1, "single_star_50_periodic": 5}.get(workload, 5)


# --------------------------------------------------------------- our arm

def record_bytes(precision):
    """Bytes of one solvent record: float4 pos + float4 vel (FP64: double4 x2)."""
    return 32 if precision == "fp32" else 64


def key_bytes(precision, specs):
    """Bytes of one sort key: the FP32 fast path packs (local cell, rank) into
    32 bits when every box has at most 65,536 cells; otherwise (global cell,
    rank) pairs of 8 bytes."""
    return 4 if precision == "fp32" and max(s.L ** 3 for s in specs) <= 65536 else 8


def kernel_rooflines(phases, cycles, n_solvent, slots, n_cells, rec, peak, kb=8):
    """Achieved HBM GB/s of the solvent kernels from their CUDA-event times
    (ms summed over ``cycles``) and their algorithmic bytes per launch (kb:
    bytes of one sort key):
      fluid_bin   read a record, write the key               (rec + kb) B / particle
      build_perm  read the key, write the 4-byte sorted entry  (kb + 4) B / entry
      collide     read the entry and the record, write the record back
                  (4 + 2 rec) B / entry + 4 B / cell (offsets)"""
    alg = {"fluid_bin": n_solvent * (rec + kb),
           "build_perm": slots * (kb + 4),
           "collide": slots * (4 + 2 * rec) + (n_cells + 1) * 4}
    out = {}
    for k, nbytes in alg.items():
        ms = phases.get(k, 0.0) / cycles
        if ms <= 0:
            continue
        gbs = nbytes / (ms / 1e3) / 1e9
        out[k] = {"achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
                  "frac": round(gbs / peak, 4), "algorithmic_bytes_per_launch": int(nbytes),
                  "launch_ms": round(ms, 4)}
    return out


def run_ours(args, world, rank, local, dist):
    from starpolymersmd_gb300 import capi, workloads as W

    prec = capi.FP32 if args.precision == "fp32" else capi.FP64
    rec = record_bytes(args.precision)
    t_build = time.perf_counter()
    if args.replicas and args.workload == "batched_256":
        built = W.batched_256(precision=prec, n=args.replicas)
    else:
        built = W.WORKLOADS[args.workload](precision=prec)
    ctx = built.ctx
    build_s = time.perf_counter() - t_build
    units = built.particles
    K, Wm = args.steps, max(3, args.warmup)
    ctx.cycles(Wm)
    # launch shapes picked by the project's autotuner (cached per GPU + workload;
    # the trial cycles run on a saved copy of the state, which is then restored)
    from starpolymersmd_gb300 import autotune
    key = autotune.signature(built.n_rep, built.particles,
                             sum(s.L ** 3 for s in built.specs), int(sum(built.n_mono)))
    key += "" if prec == capi.FP32 else "-fp64"
    tuned = autotune.tune(ctx, key, cycles=3)
    ctx.cycles(2)
    ctx.synchronize()
    ctx.raise_on_device_error()

    gpu_index = local
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        try:
            gpu_index = int(vis.split(",")[local])
        except ValueError:
            pass
    sampler = ClockSampler(gpu_index)
    sampler.start()
    # keep the GPU on the same work until the sampler's first row is in
    t_wait = time.perf_counter()
    while sampler.rows_written() == 0 and time.perf_counter() - t_wait < 5.0:
        ctx.cycles(max(1, Wm))
        ctx.synchronize()
    barrier(dist)
    ms = ctx.time_cycles(K)
    # and for about 100 ms after the timed region
    t_after = time.perf_counter()
    while time.perf_counter() - t_after < 0.1:
        ctx.cycles(max(1, Wm))
        ctx.synchronize()
    clocks = sampler.stop()
    ctx.raise_on_device_error()
    ms = max_over_ranks(dist, ms)
    barrier(dist)
    value = job_value(units, K, world, ms)
    rep_steps = built.n_rep * K * world / (ms / 1e3)

    # per-kernel device times over a second timed region (events on the stream)
    phases, tot = ctx.cycles_profiled(K)
    n_cells = sum(n * n * n for n in (s.L for s in built.specs))
    n_solvent = int(sum(built.n_fluid))
    slots = units  # every solvent particle and monomer passes the collide kernel once
    peak, peak_kind = measured_peaks()
    kb = key_bytes(args.precision, built.specs)
    per_kernel = kernel_rooflines(phases, K, n_solvent, slots, n_cells, rec, peak, kb)
    coll = per_kernel["collide"]
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath) and not args.replicas and prec == capi.FP32:
        with open(tpath) as f:
            tj = json.load(f)
        if args.workload in tj:
            traffic = tj[args.workload].get("collide_bytes_per_launch")
    roofline = {"kernel": "k_collide", "bound": "hbm", "achieved": coll["achieved"],
                "peak": peak, "unit": "GB/s", "frac": coll["frac"],
                "traffic": traffic, "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": coll["algorithmic_bytes_per_launch"],
                "launch_ms": coll["launch_ms"]}
    if prec == capi.FP64:
        roofline["note"] = ("FP64 kernels issue on the FP64 pipe (2 DFMA per clock per SM), "
                            "not HBM-bound; the HBM fraction is reported for comparison")
    phase_share = {k: round(v / tot, 4) for k, v in phases.items()} if tot > 0 else {}
    cycle_alg_bytes = units * 2 * rec + n_cells * 88
    whole = {"achieved_gbs": round(cycle_alg_bytes / (ms / K / 1e3) / 1e9, 1),
             "frac": round(cycle_alg_bytes / (ms / K / 1e3) / 1e9 / peak, 4),
             "alg_bytes_per_cycle": cycle_alg_bytes}

    launches_per_cycle = (PHASE_LAUNCHES - 1 + PMD_LAUNCHES * W.N_SUB + 2
                          if args.workload in W.PERIODIC else PHASE_LAUNCHES)
    big = sum(1 for n in built.n_mono if n > 512)
    if ctx.get_variants()[2] == 3 and 0 < big < built.n_rep:
        launches_per_cycle += 1  # the side-by-side MD shape runs two MD kernels
    precision_desc = ("fp32 state, int64 fixed-point cell sums, fp64 delrx" if prec == capi.FP32
                      else "fp64 state, the reference's operation order")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
           "warmup": Wm, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32" if prec == capi.FP32 else "f64",
           "data": "synthetic (device-drawn uniform solvent, Maxwell-Boltzmann velocities, "
                   "self-avoiding-walk stars)",
           "config": {"workload": args.workload, "replicas": built.n_rep,
                      "particles": units, "solvent": n_solvent,
                      "monomers": int(sum(built.n_mono)), "cells": n_cells,
                      "md_substeps_per_cycle": W.N_SUB, "h": W.H, "md_dt": W.MD_DT,
                      "precision": precision_desc,
                      "sort_keys": "32-bit (local cell << 16 | rank)" if kb == 4
                                   else "64-bit (global cell, rank)",
                      "l2": "state of %.1f GB per copy, %s" % (
                          units * rec / 1e9, "inputs larger than L2" if units * rec > 129e6
                          else "state fits in the 129 MB L2 (the workload's own size)"),
                      "parallelism": "replicas only" if world == 1 else f"replicas x{world}"},
           "replica_steps_per_s": rep_steps, "gpu_launches": launches_per_cycle * K,
           "autotune": {"chosen": {k: v.get("chosen") for k, v in tuned["report"].items()},
                        "cached": tuned["cached"]},
           "roofline": roofline, "kernel_rooflines": per_kernel, "cycle_roofline": whole,
           "phase_share": phase_share, "build_s": round(build_s, 1)}
    if clocks:
        out["clocks"] = clocks
    if args.workload == "single_star_50_periodic":
        # no bead may meet another bead's periodic image: the star's extent
        # along every axis stays below L - r_cut (then this is single_star_50's
        # physics through the periodic MD kernels)
        ext = W.star_extent(built)
        L = float(built.specs[0].L)
        out["config"]["star_extent_after_run"] = [round(float(e), 2) for e in ext]
        out["config"]["self_image_free"] = bool(float(ext.max()) < L - W.R_CUT_LJ)

    if not args.no_extras:
        if prec == capi.FP32:
            out["fp64_plain"] = fp64_plain_ratio(args.workload, built, rep_steps, peak)
        out["e2e"] = e2e_measure(ctx, built, K)
        if rank == 0 and world == 1:
            ncores = os.cpu_count() or 1
            v, desc, _, _ = cpu_sample(args.workload, ncores, cpu_cycles_for(args.workload, ncores))
            out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
                                   "sample": desc}
    built.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


FP64_PLAIN_SAMPLE = 32
FP64_PLAIN_CYCLES = 10


def fp64_plain_ratio(workload, built, batched_rep_steps, peak):
    """Plain FP64 GPU path: each replica of a sample in its own FP64 context
    (the drop-in's form: one system per context), one after another, timed
    for FP64_PLAIN_CYCLES cycles after warm-up; the sample is every k-th
    replica (all of them up to FP64_PLAIN_SAMPLE), and the time of one cycle of
    every replica is the sample's time scaled by n_replicas / n_sample. A
    second pass per replica gives the per-kernel split."""
    from starpolymersmd_gb300 import capi, workloads as W
    specs = built.specs
    step = max(1, -(-len(specs) // FP64_PLAIN_SAMPLE))
    sample = list(range(0, len(specs), step))[:FP64_PLAIN_SAMPLE]
    cyc = FP64_PLAIN_CYCLES
    t_sum = 0.0
    phases_sum = {}
    n_solvent = slots = n_cells = 0
    for i in sample:
        s = specs[i]
        if workload in W.SOLUTIONS:
            b = W.build_solution(s, precision=capi.FP64)
        elif workload in W.PERIODIC:
            b = W.build([s], precision=capi.FP64, flags=capi.REPLICA_PERIODIC_MD)
        else:
            b = W.build([s], precision=capi.FP64)
        b.ctx.cycles(3)
        t_sum += b.ctx.time_cycles(cyc) / 1e3
        ph, _ = b.ctx.cycles_profiled(cyc)
        for k, v in ph.items():
            phases_sum[k] = phases_sum.get(k, 0.0) + v
        b.ctx.raise_on_device_error()
        n_solvent += int(sum(b.n_fluid))
        slots += b.particles
        n_cells += s.L ** 3
        b.close()
    scale = len(specs) / len(sample)
    per_cycle_all = t_sum / cyc * scale
    plain = len(specs) / per_cycle_all
    tot = sum(phases_sum.values())
    # kernel rooflines over the sample (the launches of all sampled replicas
    # together: bytes and times summed)
    per_kernel = kernel_rooflines(phases_sum, cyc, n_solvent, slots, n_cells, record_bytes("fp64"),
                                  peak)
    return {"replica_steps_per_s": plain, "sample_replicas": len(sample),
            "replicas": len(specs), "cycles_per_replica": cyc,
            "ms_per_cycle_all_replicas": round(per_cycle_all * 1e3, 3),
            "phase_ms_per_cycle_all_replicas": {k: round(v / cyc * scale, 4)
                                                for k, v in phases_sum.items()},
            "phase_share": {k: round(v / tot, 4) for k, v in phases_sum.items()} if tot else {},
            "kernel_rooflines": per_kernel,
            "bound": "FP64 pipe (2 DFMA per clock per SM) and the dependent-load latency of "
                     "one small system per launch; HBM fractions for comparison",
            "batched_fp32_over_plain_fp64": batched_rep_steps / plain}


def e2e_measure(ctx, built, K):
    """Through the C ABI with host buffers: per cycle, upload every monomer's
    position and velocity from pinned host memory, run the cycle, read the
    monomer state and every replica's output-step observables back (gyration
    tensor, rotation frequency, polymer kinetic energy and temperature: what
    the reference driver reads after a step, star-polymers.cpp:466-473), all
    in one smpc_cycles_io call with one synchronisation."""
    import torch
    from starpolymersmd_gb300 import capi
    n = int(sum(built.n_mono))
    pos = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    vel = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    obs = torch.empty((built.n_rep, capi.OBS_PER_REP), dtype=torch.float64,
                      pin_memory=True).numpy()
    ctx.get_monomer_state_all(pos, vel)
    k = max(3, min(K, 50))
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(k):
        ctx.cycles_io(1, pos, vel, pos, vel, obs)
    dt = time.perf_counter() - t0
    ctx.raise_on_device_error()
    if not np.all(np.isfinite(obs)):
        raise RuntimeError("non-finite observables")
    h2d = n * 6 * 8  # positions + velocities, 3 doubles each
    d2h = n * 6 * 8 + built.n_rep * capi.OBS_PER_REP * 8
    return {"value": built.particles * k / dt, "unit": UNIT, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "steps": k,
            "what": "per cycle, one smpc_cycles_io call: monomer state up, cycle, monomer state "
                    "+ per-replica gyration tensor / rotation frequency / polymer temperature down"}


# ---------------------------------------------------------- reference arm

def run_reference(args, world, rank):
    """The reference's CPU path on the host cores, like for like with our arm:
    the same workload (every replica), W untimed warm-up cycles, then K timed
    cycles (K capped so the run stays within minutes). The reference compiled
    from its own sources cannot be built where its sources are absent, so this
    arm runs the oracle's C restatement of it (kind "port")."""
    if rank != 0:
        return
    ncores = os.cpu_count() or 1
    K, Wm = min(args.steps, REF_MAX_STEPS), max(3, args.warmup)
    systems, desc = cpu_systems(args.workload, ncores, all_replicas=True)
    cpu_run(systems, ncores, Wm)
    units, secs = cpu_run(systems, ncores, K)
    v = units / secs
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": K,
           "warmup": Wm, "ms_per_step": secs / K * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
           "data": "synthetic", "config": {"workload": args.workload,
                                           "particles": int(sum(u for _, u, _ in systems)),
                                           "replicas": len(systems)},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
                            "sample": desc + f", {Wm} warm-up + {K} timed cycle(s)"},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    world, rank, local, dist = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
