"""Shared set-up for the GPU tests: build systems for the CUDA path and the
CPU oracle from the same seeded inputs."""
import numpy as np

from oracle import oracle as orc
from starpolymersmd_gb300 import capi, system
from tests import golden_replay as gr

# Tolerances stated by the tests:
FP64_RTOL = 1e-12          # FP64 path vs reference / oracle, relative to the array's scale
FP32_POS_ATOL = 2e-5       # FP32 path: absolute position error per unit of box edge
FP32_VEL_RTOL = 2e-5       # FP32 path: velocity error relative to the velocity scale


def close64(gpu, ref, rtol=FP64_RTOL):
    gpu = np.asarray(gpu)
    ref = np.asarray(ref)
    scale = max(1.0, float(np.abs(ref).max()) if ref.size else 1.0)
    np.testing.assert_allclose(gpu, ref, rtol=rtol, atol=rtol * scale)


def wrapped_diff(a, b, L):
    d = np.asarray(a) - np.asarray(b)
    Lv = np.asarray(L, dtype=np.float64)
    return d - Lv * np.round(d / Lv)


def fixture_context(fx, precision=capi.FP64, periodic=False):
    """Context replaying a reference fixture; with ``periodic`` the box runs
    the periodic many-molecule MD (wrapped monomer binning), which for one
    star away from the faces is the reference's MD."""
    n_f = len(fx["fluid_pos0"])
    star = gr.has_star(fx)
    n_m = len(fx["mono_pos0"]) if star else 0
    rep = dict(L=fx["L"], n_fluid=n_f, n_mono=n_m, mol0_size=n_m, kT=float(fx["kT"]),
               shear=float(fx["shear"]), h=float(fx["h"]), md_dt=float(fx["md_dt"]),
               flags=capi.REPLICA_PERIODIC_MD if periodic else 0,
               **{"lambda": float(fx["lam"])})
    ctx = capi.Context([rep], precision=precision, rng=capi.RNG_INJECT,
                       step_update=int(fx["step_update"]),
                       mono_bin=capi.MONOBIN_WRAPPED if periodic else capi.MONOBIN_REFERENCE,
                       angular_momentum=bool(int(fx.get("amc", 0))),
                       md_thermostat=(capi.MDTHERMO_ANDERSEN if gr.is_andersen(fx)
                                      else capi.MDTHERMO_NONE),
                       andersen_nu=float(fx.get("andersen_nu", 0.0)))
    ctx.set_fluid(0, fx["fluid_pos0"], fx["fluid_vel0"])
    if star:
        ctx.set_monomers(0, fx["mono_pos0"], fx["mono_vel0"], fx["mono_force0"], fx["mono_mass"],
                         fx["mono_amphi"], fx["mono_anchor"])
        ctx.set_bonds(0, fx["bond_src"], fx["bond_dst"])
        ctx.init_md()
    return ctx


def small_star_system(L=10, n_c=10, arms=3, n_arm=6, frac=0.5, shear=0.05, seed=3,
                      mass=5.0, kT=1.0, potential=capi.POT_REF4824):
    """Seeded compact SAW star in a uniform solvent (reference velocity init).

    The star must fit the reference's box-bounded Verlet grid and its
    unwrapped monomer binning, so walks are unbiased and regrown until the
    star stays 1.5 cells inside the box."""
    rng = np.random.default_rng(seed)
    for _ in range(200):
        star = system.make_star(arms, n_arm, frac, mass, kT, rng, bond=1.01, outward_bias=0.0)
        if np.abs(star.pos).max() < L / 2 - 1.5:
            break
    else:
        raise RuntimeError("no compact star found")
    fpos, fvel = system.uniform_fluid((L, L, L), n_c, kT, rng, reference_velocities=True)
    return star, fpos, fvel


def oracle_for(star, fpos, fvel, L, kT, shear, step_update, md_dt=0.01, lam=1.0,
               potential=orc.POT_REF4824, r_cut=1.5, r_verlet=2.0):
    n_m = star.n if star is not None else 0
    o = orc.OracleSystem((L, L, L), kT, shear, step_update, len(fpos), n_m,
                         mol_start=[0, n_m] if n_m else [0], lambda_=lam, md_dt=md_dt,
                         potential=potential, r_cut=r_cut, r_verlet=r_verlet)
    o.set_fluid(fpos, fvel)
    if n_m:
        o.set_monomers(star.pos, star.vel, np.zeros_like(star.pos), np.full(n_m, star.mass),
                       star.amphi, star.anchor)
        o.set_bonds(star.bond_src, star.bond_dst)
        o.init_md()
    return o


def context_for(star, fpos, fvel, L, kT, shear, step_update, h=0.1, md_dt=0.01, lam=1.0,
                precision=capi.FP64, rng=capi.RNG_INJECT, seed=1, potential=capi.POT_REF4824,
                r_cut=1.5, r_verlet=2.0, mono_bin=capi.MONOBIN_REFERENCE, strict=None,
                delrx_mode=capi.DELRX_REFERENCE):
    n_m = star.n if star is not None else 0
    rep = dict(L=(L, L, L), n_fluid=len(fpos), n_mono=n_m, mol0_size=n_m, kT=kT, shear=shear,
               h=h, md_dt=md_dt, seed=seed, potential=potential, r_cut=r_cut,
               r_verlet=r_verlet, **{"lambda": lam})
    ctx = capi.Context([rep], precision=precision, rng=rng, step_update=step_update,
                       mono_bin=mono_bin, strict_cells=strict, delrx_mode=delrx_mode)
    ctx.set_fluid(0, fpos, fvel)
    if n_m:
        ctx.set_monomers(0, star.pos, star.vel, np.zeros_like(star.pos), np.full(n_m, star.mass),
                         star.amphi, star.anchor)
        ctx.set_bonds(0, star.bond_src, star.bond_dst)
        ctx.init_md()
    return ctx


def fp32_cycle_check(ctx, o, rep, L):
    """One cycle of the FP32 context (already run) against the oracle (run
    from the same FP32 state on the 23-bit uniforms). Returns the number of
    particles binned differently."""
    fc, mc = ctx.cell_members(rep)
    ofc, omc = o.cell_members()
    flip_f = np.flatnonzero(fc != ofc)
    flip_m = np.flatnonzero(mc != omc)
    n = len(fc) + len(mc)
    n_flip = len(flip_f) + len(flip_m)
    # a particle within FP32 rounding of a cell face (|x| ulp ~ 2e-6 here)
    # lands in the neighbouring cell with probability ~1e-5 per particle
    assert n_flip <= 5 + 5e-5 * n, n_flip
    touched = np.unique(np.concatenate([fc[flip_f], ofc[flip_f], mc[flip_m], omc[flip_m]]))
    ex_f = np.isin(fc, touched) | np.isin(ofc, touched)
    ex_m = np.isin(mc, touched) | np.isin(omc, touched)
    p, v = ctx.get_fluid(rep)
    op, ov = o.get_fluid()
    dp = np.abs(wrapped_diff(p, op, (L,) * 3)).max(axis=1)
    dv = np.abs(v - ov).max(axis=1)
    vs = float(np.abs(ov).max())
    # one FP32 step from identical inputs: positions to a few ulp of L,
    # velocities to the stated FP32 tolerance, for every particle of every
    # cell that holds the same particles on both sides
    bad = ((dp > 1e-6 * L) | (dv > FP32_VEL_RTOL * vs)) & ~ex_f
    # a gamma acceptance test within FP32 rounding of its threshold (about
    # 1e-7 per cell) would change one whole cell: at most one such cell
    bad_cells = np.unique(ofc[bad])
    assert len(bad_cells) <= 1, (len(bad_cells), dp[bad].max(), dv[bad].max())
    mp, mv, _ = ctx.get_monomers(rep)
    omp, omv, _ = o.get_monomers()
    keep = ~ex_m
    assert np.abs(wrapped_diff(mp, omp, (L,) * 3)[keep]).max(initial=0.0) < 1e-4
    assert np.abs(mv - omv)[keep].max(initial=0.0) < 1e-3
    assert abs(ctx.temperature(rep) - o.temperature()) < 1e-4
    assert ctx.delrx(rep) == o.delrx
    return n_flip


def resync_oracle(ctx, o, rep):
    # the oracle continues from the FP32 state (exact in FP64), so each cycle
    # is compared on its own
    p, v = ctx.get_fluid(rep)
    o.set_fluid(p, v)
    mp, mv, mf = ctx.get_monomers(rep)
    o.set_monomers(mp, mv, mf)
