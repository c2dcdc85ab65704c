"""ctypes bindings for the CPU oracle (test infrastructure only).

``OracleSystem`` drives the C restatement in ``smpc_oracle.c``;
``RefSystem`` drives the reference compiled from its own sources
(``refbuild/``), available only where the reference checkout exists.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD_DIR, "libsmpc_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsmpc_ref.so")
# a reference checkout beside the repository, unless SMPC_REFERENCE names one
REF_SRC_SIBLING = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

RNG_INJECT, RNG_PHILOX = 0, 1
POT_REF4824, POT_LJ126 = 0, 1


def build_oracle(force: bool = False) -> str:
    """Compiles the C restatement (gcc, -ffp-contract=off) into _build/."""
    src = os.path.join(HERE, "smpc_oracle.c")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(os.path.join(HERE, "smpc_oracle.h"))):
        return ORACLE_SO
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-std=c11", "-O3", "-ffp-contract=off", "-fPIC", "-shared",
                           "-o", tmp, src, "-lm"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_reference(ref_root: str | None = None) -> str | None:
    """Compiles the reference's own sources into _ref/ when they are present."""
    ref_root = ref_root or os.environ.get("SMPC_REFERENCE") or REF_SRC_SIBLING
    if not os.path.isdir(os.path.join(ref_root, "star-polymers", "lib")):
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "refbuild"), "REF=" + ref_root])
    return REF_SO


class OrcParams(C.Structure):
    _fields_ = [("L", C.c_int * 3), ("kT", C.c_double), ("shear", C.c_double),
                ("step_update", C.c_uint), ("angular_momentum", C.c_int),
                ("lambda_", C.c_double), ("md_dt", C.c_double), ("r_cut", C.c_double),
                ("r_verlet", C.c_double), ("potential", C.c_int),
                ("delrx_dt_scale", C.c_double), ("mono_wrap", C.c_int)]


_lib = None


def _oracle_lib():
    global _lib
    if _lib is None:
        lib = C.CDLL(build_oracle())
        P = C.c_void_p
        lib.orc_create.restype = P
        lib.orc_create.argtypes = [C.POINTER(OrcParams), C.c_long, C.c_int, C.c_int, P]
        for name, args in {
            "orc_destroy": [P], "orc_clear_error": [P],
            "orc_set_fluid": [P, P, P], "orc_get_fluid": [P, P, P],
            "orc_set_monomers": [P, P, P, P, P, P, P], "orc_get_monomers": [P, P, P, P],
            "orc_set_bonds": [P, C.c_int, P, P], "orc_init_md": [P],
            "orc_set_delrx": [P, C.c_double], "orc_set_inject": [P, P, P, P, P],
            "orc_set_philox": [P, C.c_uint64, C.c_uint64],
            "orc_mpc_step": [P, C.c_long, C.c_double], "orc_propagate": [P, C.c_int],
            "orc_run": [P, C.c_long, C.c_long, C.c_double, C.c_int],
            "orc_cell_counts": [P, P, P], "orc_philox4x32_10": [P, P, P],
            "orc_set_periodic_md": [P, C.c_double], "orc_periodic_forces": [P, C.c_int, P],
            "orc_set_andersen": [P, C.c_double, C.c_uint64],
            "orc_stage_andersen": [P, C.c_int, P, P],
            "orc_set_lowe_andersen": [P, C.c_double, C.c_double, C.c_uint64],
            "orc_set_f32_uniforms": [P, C.c_int], "orc_cell_members": [P, P, P],
        }.items():
            getattr(lib, name).argtypes = args
            getattr(lib, name).restype = None
        for name, rt in {"orc_error": C.c_int, "orc_delrx": C.c_double,
                         "orc_temperature": C.c_double, "orc_epot": C.c_double,
                         "orc_n_cells": C.c_uint, "orc_verlet_rebuilds": C.c_int,
                         "orc_collision_counter": C.c_uint64}.items():
            getattr(lib, name).argtypes = [P]
            getattr(lib, name).restype = rt
        lib.orc_philox_gamma.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_double]
        lib.orc_philox_gamma.restype = C.c_double
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def philox4x32_10(ctr, key):
    lib = _oracle_lib()
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib.orc_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def philox_gamma(seed, step, cell, shape):
    return _oracle_lib().orc_philox_gamma(seed, step, cell, shape)


class OracleSystem:
    """One system (box + molecules) held by the C restatement."""

    def __init__(self, L, kT, shear, step_update, n_fluid, n_mono=0, mol_start=(0,),
                 lambda_=1.0, md_dt=0.01, r_cut=1.5, r_verlet=2.0, potential=POT_REF4824,
                 delrx_dt_scale=1.0, mono_wrap=0, angular_momentum=0):
        self.lib = _oracle_lib()
        p = OrcParams()
        for d in range(3):
            p.L[d] = int(L[d])
        p.kT, p.shear, p.step_update = kT, shear, step_update
        p.angular_momentum = int(angular_momentum)
        p.lambda_, p.md_dt, p.r_cut, p.r_verlet = lambda_, md_dt, r_cut, r_verlet
        p.potential, p.delrx_dt_scale = potential, delrx_dt_scale
        p.mono_wrap = int(mono_wrap)
        self.L = tuple(int(x) for x in L)
        self.n_fluid, self.n_mono = int(n_fluid), int(n_mono)
        ms = np.ascontiguousarray(mol_start, dtype=np.int32)
        self.n_mol = len(ms) - 1
        self.h = C.c_void_p(self.lib.orc_create(C.byref(p), self.n_fluid, self.n_mono,
                                                self.n_mol, _p(ms)))
        self._keep = []

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    # state -----------------------------------------------------------------
    def set_fluid(self, pos, vel):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        self.lib.orc_set_fluid(self.h, _p(pos), _p(vel))

    def get_fluid(self):
        pos = np.zeros((self.n_fluid, 3))
        vel = np.zeros((self.n_fluid, 3))
        self.lib.orc_get_fluid(self.h, _p(pos), _p(vel))
        return pos, vel

    def set_monomers(self, pos, vel, force=None, mass=None, amphi=None, anchor=None):
        a = [None if x is None else np.ascontiguousarray(x, dtype=np.float64)
             for x in (pos, vel, force, mass)]
        b = [None if x is None else np.ascontiguousarray(x, dtype=np.int32) for x in (amphi, anchor)]
        self.lib.orc_set_monomers(self.h, *[_p(x) for x in a + b])

    def get_monomers(self):
        pos = np.zeros((self.n_mono, 3))
        vel = np.zeros((self.n_mono, 3))
        f = np.zeros((self.n_mono, 3))
        self.lib.orc_get_monomers(self.h, _p(pos), _p(vel), _p(f))
        return pos, vel, f

    def set_bonds(self, src, dst):
        src = np.ascontiguousarray(src, dtype=np.int32)
        dst = np.ascontiguousarray(dst, dtype=np.int32)
        self.lib.orc_set_bonds(self.h, len(src), _p(src), _p(dst))

    def set_periodic_md(self, h):
        """Periodic many-molecule MD (before init_md; needs mono_wrap=1)."""
        self.lib.orc_set_periodic_md(self.h, float(h))

    def set_andersen(self, nu, seed):
        """Andersen stochastic thermostat after every MD step."""
        self.lib.orc_set_andersen(self.h, float(nu), int(seed))

    def set_lowe_andersen(self, nu, radius, seed):
        """Lowe-Andersen pair thermostat after the forces of every MD step."""
        self.lib.orc_set_lowe_andersen(self.h, float(nu), float(radius), int(seed))

    def stage_andersen(self, mono, vel):
        """Velocity resets of the next MD step in place of the Philox draws:
        monomer ``mono[k]`` gets ``vel[k]`` after the second half kick."""
        mono = np.ascontiguousarray(mono, dtype=np.int32)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
        self._keep_andersen = (mono, vel)
        self.lib.orc_stage_andersen(self.h, len(mono), _p(mono), _p(vel))

    def periodic_forces(self, grid):
        out = np.zeros((self.n_mono, 3))
        self.lib.orc_periodic_forces(self.h, int(grid), _p(out))
        return out

    def init_md(self):
        self.lib.orc_init_md(self.h)

    @property
    def delrx(self):
        return self.lib.orc_delrx(self.h)

    @delrx.setter
    def delrx(self, d):
        self.lib.orc_set_delrx(self.h, d)

    def error(self):
        return self.lib.orc_error(self.h)

    # rng -------------------------------------------------------------------
    def set_inject(self, shift, gamma, u_phi, u_theta):
        arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (shift, gamma, u_phi, u_theta)]
        self._keep = arrs
        self.lib.orc_set_inject(self.h, *[_p(x) for x in arrs])

    def set_philox(self, seed, counter=0):
        self.lib.orc_set_philox(self.h, seed, counter)

    def set_f32_uniforms(self, on=True):
        """Collision draws from the FP32 path's 23-bit uniforms."""
        self.lib.orc_set_f32_uniforms(self.h, int(on))

    @property
    def collision_counter(self):
        return self.lib.orc_collision_counter(self.h)

    # stepping --------------------------------------------------------------
    def mpc_step(self, t, dt):
        self.lib.orc_mpc_step(self.h, t, dt)

    def propagate(self, calc_epot=False):
        self.lib.orc_propagate(self.h, int(calc_epot))

    def run(self, t0, n, mpc_dt, with_md=True):
        self.lib.orc_run(self.h, t0, n, mpc_dt, int(with_md))

    # observables -----------------------------------------------------------
    def temperature(self):
        return self.lib.orc_temperature(self.h)

    def epot(self):
        return self.lib.orc_epot(self.h)

    def cell_counts(self):
        n = self.lib.orc_n_cells(self.h)
        tot = np.zeros(n, dtype=np.uint32)
        fl = np.zeros(n, dtype=np.uint32)
        self.lib.orc_cell_counts(self.h, _p(tot), _p(fl))
        return tot, fl

    def verlet_rebuilds(self):
        return self.lib.orc_verlet_rebuilds(self.h)

    def cell_members(self):
        """(fluid_cell[n_fluid], mono_cell[n_mono]) of the last collision, -1: not binned."""
        fc = np.zeros(self.n_fluid, dtype=np.int32)
        mc = np.zeros(max(self.n_mono, 1), dtype=np.int32)
        self.lib.orc_cell_members(self.h, _p(fc), _p(mc))
        return fc, mc[:self.n_mono]


def profile_bins(L, width):
    """Bins k = floor(p / width) for p in [-L/2, L/2]: floor(L/2w) - floor(-L/2w) + 1."""
    import math
    return int(math.floor(L / (2.0 * width)) - math.floor(-L / (2.0 * width)) + 1)


class RefSystem:
    """The reference's own classes (Box, MPC, Thermostat_None) via the harness."""

    TAPE_UNIFORM, TAPE_GAMMA = 1, 2

    def __init__(self, L, kT, lambda_, n_c, shear, step_update, amc=False):
        if not os.path.exists(REF_SO):
            if build_reference() is None:
                raise FileNotFoundError("reference checkout not available")
        lib = C.CDLL(REF_SO)
        P = C.c_void_p
        lib.ref_create.restype = P
        lib.ref_create.argtypes = [C.c_int] * 3 + [C.c_double, C.c_double, C.c_int, C.c_double,
                                                   C.c_uint, C.c_int]
        for name, args in {
            "ref_destroy": [P], "ref_box_size": [P, P],
            "ref_add_star": [P, C.c_uint, C.c_uint, C.c_uint, C.c_double],
            "ref_make_thermostat": [P, C.c_double], "ref_mpc_initialize": [P],
            "ref_make_andersen": [P, C.c_double, C.c_double, C.c_double],
            "ref_get_fluid": [P, P, P], "ref_set_fluid": [P, P, P],
            "ref_get_monomers": [P, P, P, P, P, P, P], "ref_set_monomers": [P, P, P],
            "ref_propagate": [P, C.c_int], "ref_mpc_step": [P, C.c_long, C.c_double],
            "ref_cell_counts": [P, P, P], "ref_cell_index": [P, P, P],
            "ref_set_delrx": [P, C.c_double],
            "ref_gyration": [P, P], "ref_run": [P, C.c_long, C.c_long, C.c_double, C.c_int],
            "ref_observables": [P, P],
            "ref_velocity_profile": [P, C.c_double, P, C.c_int, P, C.c_int],
            "ref_shift_arg_order": [P], "rand_tape_enable": [C.c_int], "rand_tape_clear": [],
            "ref_fourier_start": [P, C.c_uint, C.c_double, C.c_double],
            "ref_fourier_sample": [P], "ref_fourier_dump": [P, P, P, P],
            "ref_vacf_start": [P, C.c_uint, C.c_double], "ref_vacf_sample": [P],
            "ref_vacf_dump": [P, P, P],
            "ref_make_lowe_andersen": [P, C.c_double, C.c_double, C.c_double, C.c_double],
            "rand_tape_copy": [P, P, C.c_long], "rand_tape_reseed": [C.c_ulonglong],
        }.items():
            getattr(lib, name).argtypes = args
            getattr(lib, name).restype = None
        for name, rt in {"ref_n_fluid": C.c_long, "ref_n_mono": C.c_int,
                         "ref_n_cells": C.c_uint, "ref_delrx": C.c_double,
                         "ref_temperature": C.c_double, "ref_epot": C.c_double}.items():
            getattr(lib, name).argtypes = [P]
            getattr(lib, name).restype = rt
        lib.ref_get_bonds.argtypes = [P, P, P]
        lib.ref_get_bonds.restype = C.c_int
        for name, args in {"ref_print_fluid_complete": [P, C.c_char_p],
                           "ref_print_pdb_with_velocity": [P, C.c_char_p, C.c_int]}.items():
            getattr(lib, name).argtypes = args
            getattr(lib, name).restype = C.c_int
        lib.ref_mpc_initialize_from_file.argtypes = [P, C.c_char_p, C.c_int, C.c_int, C.c_int]
        lib.ref_mpc_initialize_from_file.restype = None
        lib.ref_star_from_file.argtypes = [P, C.c_int, C.c_char_p, C.c_uint, C.c_uint, C.c_uint,
                                           C.c_int]
        lib.ref_star_from_file.restype = None
        lib.rand_tape_size.argtypes = []
        lib.rand_tape_size.restype = C.c_long
        self.lib = lib
        self.h = C.c_void_p(lib.ref_create(L[0], L[1], L[2], kT, lambda_, n_c, shear,
                                           step_update, int(amc)))
        Lb = np.zeros(3, dtype=np.int32)
        lib.ref_box_size(self.h, _p(Lb))
        self.L = tuple(int(x) for x in Lb)

    def shift_order(self):
        o = np.zeros(3, dtype=np.int32)
        self.lib.ref_shift_arg_order(_p(o))
        return o

    @property
    def n_fluid(self):
        return self.lib.ref_n_fluid(self.h)

    @property
    def n_mono(self):
        return self.lib.ref_n_mono(self.h)

    @property
    def n_cells(self):
        return self.lib.ref_n_cells(self.h)

    def add_star(self, A, B, arms, mass):
        self.lib.ref_add_star(self.h, A, B, arms, mass)

    # the reference's restart files, through its own writers and readers
    def print_fluid_complete(self, path):
        if self.lib.ref_print_fluid_complete(self.h, os.fsencode(path)):
            raise OSError(path)

    def initialize_fluid_from_file(self, path, L_old):
        self.lib.ref_mpc_initialize_from_file(self.h, os.fsencode(path), *[int(x) for x in L_old])

    def print_pdb_with_velocity(self, path, step):
        if self.lib.ref_print_pdb_with_velocity(self.h, os.fsencode(path), int(step)):
            raise OSError(path)

    def star_from_file(self, mol, path, A, B, arms, set_zero=False):
        self.lib.ref_star_from_file(self.h, int(mol), os.fsencode(path), A, B, arms, int(set_zero))

    def make_thermostat(self, dt):
        self.lib.ref_make_thermostat(self.h, dt)

    def make_andersen(self, dt, T, nu):
        """AndersenStochastic{box, dt, T, nu} as the propagating thermostat."""
        self.lib.ref_make_andersen(self.h, dt, T, nu)

    def make_lowe_andersen(self, dt, T, nu, r):
        """Lowe_Andersen{box, dt, T, nu, r} as the propagating thermostat."""
        self.lib.ref_make_lowe_andersen(self.h, dt, T, nu, r)

    def mpc_initialize(self):
        self.lib.ref_mpc_initialize(self.h)

    def get_fluid(self):
        n = self.n_fluid
        pos, vel = np.zeros((n, 3)), np.zeros((n, 3))
        self.lib.ref_get_fluid(self.h, _p(pos), _p(vel))
        return pos, vel

    def set_fluid(self, pos, vel):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        self.lib.ref_set_fluid(self.h, _p(pos), _p(vel))

    def get_monomers(self):
        n = self.n_mono
        pos, vel, f = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        mass = np.zeros(n)
        amphi = np.zeros(n, dtype=np.int32)
        anchor = np.zeros(n, dtype=np.int32)
        self.lib.ref_get_monomers(self.h, _p(pos), _p(vel), _p(f), _p(mass), _p(amphi), _p(anchor))
        return dict(pos=pos, vel=vel, force=f, mass=mass, amphi=amphi, anchor=anchor)

    def set_monomers(self, pos, vel):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        self.lib.ref_set_monomers(self.h, _p(pos), _p(vel))

    def bonds(self):
        n = self.lib.ref_get_bonds(self.h, None, None)
        src = np.zeros(n, dtype=np.int32)
        dst = np.zeros(n, dtype=np.int32)
        self.lib.ref_get_bonds(self.h, _p(src), _p(dst))
        return src, dst

    def propagate(self, calc_epot=False):
        self.lib.ref_propagate(self.h, int(calc_epot))

    def mpc_step(self, t, dt):
        self.lib.ref_mpc_step(self.h, t, dt)

    def run(self, t0, n, mpc_dt, with_md=True):
        self.lib.ref_run(self.h, t0, n, mpc_dt, int(with_md))

    def cell_counts(self):
        n = self.n_cells
        tot = np.zeros(n, dtype=np.uint32)
        fl = np.zeros(n, dtype=np.uint32)
        self.lib.ref_cell_counts(self.h, _p(tot), _p(fl))
        return tot, fl

    def observables(self):
        """R_g, G (row-major), rotation frequency, kinetic energy, temperature, molecules."""
        out = np.zeros(16)
        self.lib.ref_observables(self.h, _p(out))
        return out

    def velocity_profile(self, width):
        """VelocityX sums (v_x, v_y, count) per bin along x and along y."""
        nx, ny = profile_bins(self.L[0], width), profile_bins(self.L[1], width)
        xo, yo = np.zeros((nx, 3)), np.zeros((ny, 3))
        self.lib.ref_velocity_profile(self.h, width, _p(xo), nx, _p(yo), ny)
        return xo, yo

    def cell_index(self):
        """CellIndex of every solvent particle and monomer at the last sort."""
        fc = np.zeros(self.n_fluid, dtype=np.int32)
        mc = np.zeros(self.n_mono, dtype=np.int32)
        self.lib.ref_cell_index(self.h, _p(fc), _p(mc))
        return fc, mc

    @property
    def delrx(self):
        return self.lib.ref_delrx(self.h)

    def temperature(self):
        return self.lib.ref_temperature(self.h)

    def epot(self):
        return self.lib.ref_epot(self.h)

    def gyration(self):
        out = np.zeros(10)
        self.lib.ref_gyration(self.h, _p(out))
        return out

    # analyses ----------------------------------------------------------------
    def fourier_start(self, entries, dt, L):
        self._fourier_entries = int(entries)
        self.lib.ref_fourier_start(self.h, int(entries), float(dt), float(L))

    def fourier_sample(self):
        self.lib.ref_fourier_sample(self.h)

    def fourier_dump(self):
        """(last sample's modes (3, 3) complex, Autocorrelation (3, entries), counter)."""
        m = np.zeros(18)
        acf = np.zeros(3 * self._fourier_entries)
        n = C.c_uint()
        self.lib.ref_fourier_dump(self.h, _p(m), _p(acf), C.byref(n))
        return (m[0::2] + 1j * m[1::2]).reshape(3, 3), acf.reshape(3, -1), n.value

    def vacf_start(self, entries, dt):
        self._vacf_entries = int(entries)
        self.lib.ref_vacf_start(self.h, int(entries), float(dt))

    def vacf_sample(self):
        self.lib.ref_vacf_sample(self.h)

    def vacf_dump(self):
        """(Autocorrelation summed over particles per lag, counter)."""
        s = np.zeros(self._vacf_entries)
        n = C.c_uint()
        self.lib.ref_vacf_dump(self.h, _p(s), C.byref(n))
        return s, n.value

    # tape ------------------------------------------------------------------
    def tape_start(self):
        self.lib.rand_tape_clear()
        self.lib.rand_tape_enable(1)

    def tape_take(self):
        n = self.lib.rand_tape_size()
        vals = np.zeros(n)
        kinds = np.zeros(n, dtype=np.int32)
        self.lib.rand_tape_copy(_p(vals), _p(kinds), n)
        self.lib.rand_tape_clear()
        return vals, kinds

    def reseed(self, seed):
        self.lib.rand_tape_reseed(seed)


def decode_andersen_tape(vals, kinds, masses, nu_dt, sigma):
    """Velocity resets of one AndersenStochastic::propagate from its draws.

    Draw order of Andersen_stochastic.cpp:49-58: for every monomer in
    molecule order one uniform; when it is below nu * dt, three normals
    N(0, sigma) (mass 1) or N(0, sigma / sqrt(m)) for x, y, z, each formed as
    Rand::real_normal(mean, std) does (Rand.cpp:16-18: z * std + mean).
    Returns (monomer indices, velocities[n, 3]).
    """
    idx, vel = [], []
    k = 0
    for i, m in enumerate(masses):
        assert kinds[k] == 1, "expected the trigger uniform"
        u = vals[k]
        k += 1
        if u < nu_dt:
            assert all(kinds[k + d] == 3 for d in range(3)), "expected three normals"
            std = sigma if m == 1.0 else sigma / np.sqrt(m)
            vel.append([vals[k + d] * std + 0.0 for d in range(3)])
            idx.append(i)
            k += 3
    assert k == len(vals), (k, len(vals))
    return np.array(idx, dtype=np.int32), np.array(vel, dtype=np.float64).reshape(-1, 3)


def decode_collision_tape(vals, kinds, counts, shift_order):
    """Splits the draws of one collision into (shift[3], gamma, u_phi, u_theta).

    Draw order of MPC::step (MPC.cpp:123-138): three uniforms for the grid
    shift (assigned to components per ``shift_order``), then for every cell in
    index order a gamma variate if the cell holds >= 2 particles
    (MPC.cpp:287-289) followed by the uniforms for phi and theta
    (MPC.cpp:244-245). ``gamma`` is NaN where no variate was drawn.
    """
    n_cell = len(counts)
    assert kinds[0] == 1 and kinds[1] == 1 and kinds[2] == 1
    draws = vals[:3] - 0.5
    shift = np.array([draws[shift_order[0]], draws[shift_order[1]], draws[shift_order[2]]])
    gamma = np.full(n_cell, np.nan)
    u_phi = np.zeros(n_cell)
    u_th = np.zeros(n_cell)
    k = 3
    for c in range(n_cell):
        if counts[c] >= 2:
            assert kinds[k] == 2, "expected a gamma draw"
            gamma[c] = vals[k]
            k += 1
        assert kinds[k] == 1 and kinds[k + 1] == 1
        u_phi[c] = vals[k]
        u_th[c] = vals[k + 1]
        k += 2
    assert k == len(vals), (k, len(vals))
    return shift, gamma, u_phi, u_th
