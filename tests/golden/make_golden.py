"""Generates the golden fixtures in this directory from the reference itself.

Each fixture runs the StarPolymersMD reference -- its own sources, compiled
unmodified by oracle/refbuild against a project-written Eigen subset and a
recording Rand.cpp -- at library level, and stores:

* the parameters and the initial state (fluid, monomers incl. forces, bonds);
* for every collision: the grid shift and the per-cell gamma / phi / theta
  draws decoded from the reference's own mt19937_64 stream, plus the cell
  occupancies after MPC::sort (total and fluid-only);
* the state after every driver-loop iteration for monomers, and the fluid
  state after every collision (small boxes only), the fluid temperature and
  the Lees-Edwards offset.

Run from the repository root where the reference checkout exists:
    python tests/golden/make_golden.py [--ref /path/to/StarPolymersMD]
The fixtures are plain .npz files; tests read them without the reference.
"""
from __future__ import annotations

import argparse
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from starpolymersmd_gb300 import system  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
PROFILE_WIDTH = 0.2  # VelocityX bin width of star-polymers.cpp:355

SCENARIOS = {
    # pure solvent with Lees-Edwards shear, like mpc_test.cpp (step_update = 1)
    "mpc_shear_L6": dict(L=(6, 6, 6), n_c=10, kT=1.0, shear=0.1, step_update=1, h=0.1,
                         star=None, n_loop=4, with_md=False),
    # pure solvent, no shear: plain periodic wrap branch (MPC.cpp:473-478)
    "mpc_noshear_L4": dict(L=(4, 4, 4), n_c=5, kT=0.5, shear=0.0, step_update=1, h=0.1,
                           star=None, n_loop=3, with_md=False),
    # star + solvent, 10 MD substeps per collision, delrx over-advance quirk
    "star_mpc_L12": dict(L=(12, 12, 12), n_c=3, kT=1.0, shear=0.05, step_update=10, h=0.1,
                         md_dt=0.01, lam=1.0, star=dict(A=2, B=2, arms=3, mass=5.0),
                         n_loop=26, with_md=True),
    # star pushed toward the box edge: MPC::check_bounds recentres everything
    "recentre_L12": dict(L=(12, 12, 12), n_c=3, kT=1.0, shear=0.05, step_update=1, h=0.1,
                         md_dt=0.01, lam=1.0, star=dict(A=2, B=2, arms=3, mass=5.0),
                         n_loop=3, with_md=True, star_offset=(3.5, -1.0, 0.5)),
    # the angular-momentum-conserving collision (MPC.cpp:260-269, 324-374)
    "amc_mpc_L6": dict(L=(6, 6, 6), n_c=6, kT=1.0, shear=0.1, step_update=1, h=0.1,
                       star=None, n_loop=3, with_md=False, amc=True),
    "amc_star_L12": dict(L=(12, 12, 12), n_c=3, kT=1.0, shear=0.05, step_update=5, h=0.1,
                         md_dt=0.01, lam=1.0, star=dict(A=2, B=2, arms=3, mass=5.0),
                         n_loop=11, with_md=True, amc=True),
    # larger self-avoiding star, MD only with a strong BB attraction
    "md_saw_L16": dict(L=(16, 16, 16), n_c=1, kT=1.0, shear=0.0, step_update=1, h=0.1,
                       md_dt=0.01, lam=1.5, star=dict(A=5, B=5, arms=6, mass=5.0),
                       saw_seed=7, n_loop=60, with_md=True, md_only=True),
    # MPC off: the driver's AndersenStochastic integrator (star-polymers.cpp:387),
    # heavy monomers (N(0, sqrt(T / m)) resets) and unit-mass ones (N(0, sqrt(T)))
    "andersen_saw_L16": dict(L=(16, 16, 16), n_c=1, kT=1.0, shear=0.0, step_update=1, h=0.1,
                             md_dt=0.01, lam=1.5, star=dict(A=5, B=5, arms=6, mass=5.0),
                             saw_seed=11, n_loop=60, with_md=True, md_only=True,
                             andersen_nu=2.0),
    "andersen_m1_L12": dict(L=(12, 12, 12), n_c=1, kT=0.8, shear=0.0, step_update=1, h=0.1,
                            md_dt=0.005, lam=1.0, star=dict(A=2, B=2, arms=3, mass=1.0),
                            n_loop=40, with_md=True, md_only=True, andersen_nu=5.0),
    # the reference's solvent analyses, Fourier_Autocorr and Vel_Autocorr_Fluid
    # over every solvent particle, sampled after every collision of a sheared
    # solvent (windows of 3 and 4 samples)
    "analysis_L6": dict(L=(6, 6, 6), n_c=5, kT=1.0, shear=0.2, step_update=1, h=0.1,
                        star=None, n_loop=9, with_md=False, analysis=(3, 4)),
}


def run_scenario(name: str, sc: dict) -> dict:
    ref = orc.RefSystem(sc["L"], sc["kT"], sc.get("lam", 1.0), sc["n_c"], sc["shear"],
                        sc["step_update"], amc=sc.get("amc", False))
    ref.reseed(1)
    order = ref.shift_order()
    st = sc.get("star")
    if st:
        ref.add_star(st["A"], st["B"], st["arms"], st["mass"])
        mono = ref.get_monomers()
        if "saw_seed" in sc:
            rng = np.random.default_rng(sc["saw_seed"])
            pos = system.saw_star(st["arms"], st["A"] + st["B"], rng, bond=1.01)
            pos -= pos.mean(axis=0)
            ref.set_monomers(pos, mono["vel"])
        if "star_offset" in sc:
            ref.set_monomers(mono["pos"] + np.asarray(sc["star_offset"]), mono["vel"])
        if "andersen_nu" in sc:
            ref.make_andersen(sc["md_dt"], sc["kT"], sc["andersen_nu"])
        else:
            ref.make_thermostat(sc["md_dt"])
    if not sc.get("md_only"):
        ref.mpc_initialize()
    fpos0, fvel0 = ref.get_fluid()
    m0 = ref.get_monomers() if st else None
    src, dst = ref.bonds() if st else (np.zeros(0, np.int32), np.zeros(0, np.int32))
    out = dict(L=np.array(ref.L, dtype=np.int32), n_c=sc["n_c"], kT=sc["kT"], shear=sc["shear"],
               step_update=sc["step_update"], h=sc["h"], md_dt=sc.get("md_dt", 0.0),
               lam=sc.get("lam", 1.0), n_loop=sc["n_loop"], with_md=int(sc["with_md"]),
               md_only=int(bool(sc.get("md_only"))), shift_order=order,
               amc=int(bool(sc.get("amc"))),
               fluid_pos0=fpos0, fluid_vel0=fvel0, bond_src=src, bond_dst=dst)
    if st:
        out.update(mono_pos0=m0["pos"], mono_vel0=m0["vel"], mono_force0=m0["force"],
                   mono_mass=m0["mass"], mono_amphi=m0["amphi"], mono_anchor=m0["anchor"])
    shifts, gammas, uphis, uths, tots, fls, steps = [], [], [], [], [], [], []
    fl_pos, fl_vel, temps, fl_cell, mo_cell = [], [], [], [], []
    obs, prof_x, prof_y = [], [], []
    m_pos, m_vel, m_frc, delrx, epots = [], [], [], [], []
    and_start, and_idx, and_vel = [0], [], []
    modes = []
    if "analysis" in sc:
        ref.fourier_start(sc["analysis"][0], sc["h"], ref.L[0])
        ref.vacf_start(sc["analysis"][1], sc["h"])
    for t in range(sc["n_loop"]):
        if st and sc["with_md"]:
            if "andersen_nu" in sc:
                ref.tape_start()
            ref.propagate(True)
            if "andersen_nu" in sc:
                vals, kinds = ref.tape_take()
                ix, vv = orc.decode_andersen_tape(vals, kinds, m0["mass"],
                                                  sc["andersen_nu"] * sc["md_dt"],
                                                  math.sqrt(sc["kT"]))
                and_idx.append(ix); and_vel.append(vv)
                and_start.append(and_start[-1] + len(ix))
            epots.append(ref.epot())
        if not sc.get("md_only"):
            ref.tape_start()
            ref.mpc_step(t, sc["h"])
            vals, kinds = ref.tape_take()
            if len(vals):
                tot, fl = ref.cell_counts()
                s, g, up, ut = orc.decode_collision_tape(vals, kinds, tot, order)
                shifts.append(s); gammas.append(g); uphis.append(up); uths.append(ut)
                tots.append(tot); fls.append(fl); steps.append(t)
                p, v = ref.get_fluid()
                fl_pos.append(p); fl_vel.append(v)
                temps.append(ref.temperature())
                fc, mc = ref.cell_index()
                fl_cell.append(fc); mo_cell.append(mc)
                if "analysis" in sc:
                    ref.fourier_sample()
                    modes.append(ref.fourier_dump()[0])
                    ref.vacf_sample()
                if st:
                    # output-step observables (star-polymers.cpp:467-473, 483)
                    obs.append(ref.observables())
                    px, py = ref.velocity_profile(PROFILE_WIDTH)
                    prof_x.append(px); prof_y.append(py)
        delrx.append(ref.delrx)
        if st:
            m = ref.get_monomers()
            m_pos.append(m["pos"]); m_vel.append(m["vel"]); m_frc.append(m["force"])
    out.update(coll_steps=np.array(steps, dtype=np.int64), delrx=np.array(delrx),
               epot=np.array(epots))
    if "andersen_nu" in sc:
        # per driver-loop step t: monomers and_idx[and_start[t]:and_start[t + 1]]
        # got the velocities and_vel[...] from the reference's draws
        out.update(andersen_nu=sc["andersen_nu"],
                   andersen_start=np.array(and_start, dtype=np.int32),
                   andersen_idx=np.concatenate(and_idx).astype(np.int32),
                   andersen_vel=np.concatenate(and_vel).reshape(-1, 3))
    if steps:
        out.update(shift=np.array(shifts), gamma=np.array(gammas), u_phi=np.array(uphis),
                   u_theta=np.array(uths), count_total=np.array(tots), count_fluid=np.array(fls),
                   fluid_pos=np.array(fl_pos), fluid_vel=np.array(fl_vel),
                   temperature=np.array(temps), fluid_cell=np.array(fl_cell),
                   mono_cell=np.array(mo_cell))
        if obs:
            out.update(observables=np.array(obs), profile_x=np.array(prof_x),
                       profile_y=np.array(prof_y), profile_width=PROFILE_WIDTH)
    if st:
        out.update(mono_pos=np.array(m_pos), mono_vel=np.array(m_vel), mono_force=np.array(m_frc),
                   gyration=ref.gyration())
    if "analysis" in sc:
        _, acf, n_f = ref.fourier_dump()
        sums, n_v = ref.vacf_dump()
        out.update(fourier_entries=sc["analysis"][0], fourier_modes=np.array(modes),
                   fourier_acf=acf, fourier_counter=n_f, vacf_entries=sc["analysis"][1],
                   vacf_lag_sums=sums, vacf_counter=n_v)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    if orc.build_reference(args.ref) is None:
        sys.exit("reference checkout not found")
    for name, sc in SCENARIOS.items():
        if args.only and name != args.only:
            continue
        data = run_scenario(name, sc)
        path = os.path.join(OUT, name + ".npz")
        np.savez_compressed(path, **data)
        print(f"{name}: {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
