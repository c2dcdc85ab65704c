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
                 "-lms", "200", "-i", str(self.gpu)], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

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
                "samples": len(rows)}


# ------------------------------------------------------------ CPU baseline

def cpu_sample(workload, n_threads, cycles, max_replicas=None):
    """The oracle (C restatement of the reference, FP64) on host cores: one
    replica per thread, ``cycles`` cycles each. Returns (units/s, description)."""
    from oracle import oracle as orc
    from starpolymersmd_gb300 import system, workloads as W

    if workload in W.SOLUTIONS:
        pick = [W.SOLUTION_SPECS[workload]()]
    elif workload == "batched_256":
        specs = system.batched_replica_table(256)
        pick = specs[:: max(1, len(specs) // n_threads)][:n_threads]
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
        return o, n_f + st.n

    systems = [make(s) for s in pick]

    def run(item):
        o, units = item
        o.run(1, W.N_SUB * cycles, W.H, True)  # t = 1..: collisions every N_SUB calls
        return units * cycles

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=n_threads) as ex:
        done = sum(ex.map(run, systems))
    dt = time.perf_counter() - t0
    desc = (f"oracle C restatement (FP64), {len(systems)} replica(s) of {workload} "
            f"({', '.join(f'L={s.L}' for s in pick[:6])}{'...' if len(pick) > 6 else ''}), "
            f"{cycles} cycle(s) each, one replica per thread")
    return done / dt, desc, done, dt


def cpu_cycles_for(workload, n_threads):
    # about 10-30 s of CPU work in total
    return {"batched_256": 20, "single_star_50": 5, "single_star_20": 40, "semidilute_100": 3,
            "large_box_200": 1, "single_star_50_periodic": 5}.get(workload, 5)


# --------------------------------------------------------------- our arm

def run_ours(args, world, rank, local, dist):
    from starpolymersmd_gb300 import capi, workloads as W

    t_build = time.perf_counter()
    if args.replicas and args.workload == "batched_256":
        built = W.batched_256(precision=capi.FP32, n=args.replicas)
    else:
        built = W.WORKLOADS[args.workload](precision=capi.FP32)
    ctx = built.ctx
    build_s = time.perf_counter() - t_build
    units = built.particles
    K, Wm = args.steps, max(3, args.warmup)
    ctx.cycles(Wm)
    # launch shapes picked by the project's autotuner (cached per GPU + workload)
    from starpolymersmd_gb300 import autotune
    key = autotune.signature(built.n_rep, built.particles,
                             sum(s.L ** 3 for s in built.specs), int(sum(built.n_mono)))
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
    barrier(dist)
    sampler.start()
    ms = ctx.time_cycles(K)
    clocks = sampler.stop()
    ctx.raise_on_device_error()
    ms = max_over_ranks(dist, ms)
    barrier(dist)
    value = job_value(units, K, world, ms)
    rep_steps = built.n_rep * K * world / (ms / 1e3)

    # per-kernel device times over a second timed region (events on the stream)
    phases, tot = ctx.cycles_profiled(K)
    n_cells = sum(n * n * n for n in (s.L for s in built.specs))
    slots = units  # every solvent particle and monomer passes the collide kernel once
    coll_ms = phases["collide"] / K
    coll_bytes = slots * (16 + 16 + 16 + 16 + 4) + (n_cells + 1) * 4
    peak, peak_kind = measured_peaks()
    achieved = coll_bytes / (coll_ms / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath) and not args.replicas:
        with open(tpath) as f:
            tj = json.load(f)
        if args.workload in tj:
            traffic = tj[args.workload].get("collide_bytes_per_launch")
    roofline = {"kernel": "k_collide", "bound": "hbm", "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": traffic, "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": coll_bytes,
                "launch_ms": round(coll_ms, 4)}
    phase_share = {k: round(v / tot, 4) for k, v in phases.items()} if tot > 0 else {}
    cycle_alg_bytes = units * 64 + n_cells * 88
    whole = {"achieved_gbs": round(cycle_alg_bytes / (ms / K / 1e3) / 1e9, 1),
             "frac": round(cycle_alg_bytes / (ms / K / 1e3) / 1e9 / peak, 4),
             "alg_bytes_per_cycle": cycle_alg_bytes}

    launches_per_cycle = (PHASE_LAUNCHES - 1 + PMD_LAUNCHES * W.N_SUB + 2
                          if args.workload in W.PERIODIC else PHASE_LAUNCHES)
    big = sum(1 for n in built.n_mono if n > 512)
    if ctx.get_variants()[2] == 3 and 0 < big < built.n_rep:
        launches_per_cycle += 1  # the side-by-side MD shape runs two MD kernels
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
           "warmup": Wm, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (device-drawn uniform solvent, Maxwell-Boltzmann velocities, "
                   "self-avoiding-walk stars)",
           "config": {"workload": args.workload, "replicas": built.n_rep,
                      "particles": units, "solvent": int(sum(built.n_fluid)),
                      "monomers": int(sum(built.n_mono)), "cells": n_cells,
                      "md_substeps_per_cycle": W.N_SUB, "h": W.H, "md_dt": W.MD_DT,
                      "precision": "fp32 state, int64 fixed-point cell sums, fp64 delrx",
                      "l2": "state of %.1f GB per copy, inputs larger than L2" % (units * 32 / 1e9),
                      "parallelism": "replicas only" if world == 1 else f"replicas x{world}"},
           "replica_steps_per_s": rep_steps, "gpu_launches": launches_per_cycle * K,
           "autotune": {"chosen": {k: v.get("chosen") for k, v in tuned["report"].items()},
                        "cached": tuned["cached"]},
           "roofline": roofline, "cycle_roofline": whole, "phase_share": phase_share,
           "build_s": round(build_s, 1)}
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
        out["fp64_plain"] = fp64_plain_ratio(args.workload, built, rep_steps)
        out["e2e"] = e2e_measure(ctx, built, K)
        if rank == 0 and world == 1:
            ncores = os.cpu_count() or 1
            v, desc, _, _ = cpu_sample(args.workload, ncores, cpu_cycles_for(args.workload, ncores))
            out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
                                   "sample": desc}
    built.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


def fp64_plain_ratio(workload, built, batched_rep_steps):
    """Plain FP64 GPU path: each replica of a sample in its own FP64 context,
    one after another; replica-steps/s of the full set estimated from the sample."""
    from starpolymersmd_gb300 import capi, workloads as W
    specs = built.specs
    step = max(1, len(specs) // 16)
    sample = specs[::step][:16]
    cyc = 3
    t_sum = 0.0
    for s in sample:
        if workload in W.SOLUTIONS:
            b = W.build_solution(s, precision=capi.FP64)
        elif workload in W.PERIODIC:
            b = W.build([s], precision=capi.FP64, flags=capi.REPLICA_PERIODIC_MD)
        else:
            b = W.build([s], precision=capi.FP64)
        b.ctx.cycles(2)
        t_sum += b.ctx.time_cycles(cyc) / 1e3
        b.ctx.raise_on_device_error()
        b.close()
    # time for one cycle of every replica, one after another
    per_cycle_all = t_sum / cyc * (len(specs) / len(sample))
    plain = len(specs) / per_cycle_all
    return {"replica_steps_per_s": plain, "sample_replicas": len(sample), "cycles": cyc,
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
    if rank != 0:
        return
    ncores = os.cpu_count() or 1
    K, Wm = args.steps, max(3, args.warmup)
    # warm-up and timed samples on the same systems; each step = one cycle of
    # one replica per core, bounded so the whole run takes a few minutes
    K = min(K, 20)
    v_w, _, _, _ = cpu_sample(args.workload, ncores, 1)
    v, desc, units, secs = cpu_sample(args.workload, ncores, K)
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": K,
           "warmup": 1, "ms_per_step": secs / K * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
           "data": "synthetic", "config": {"workload": args.workload},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
                            "sample": desc},
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
