"""ctypes binding of the C ABI in include/smpc.h (libsmpc.so).

The library is the product path: there is no CPU fallback. Importing this
module does not need a GPU; creating a context does, and any failure of the
CUDA library raises ``SmpcError``.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsmpc.so")

FP64, FP32 = 0, 1
RNG_INJECT, RNG_PHILOX = 0, 1
POT_REF4824, POT_LJ126 = 0, 1
MONOBIN_REFERENCE, MONOBIN_WRAPPED = 0, 1
DELRX_REFERENCE, DELRX_PHYSICAL = 0, 1
MDTHERMO_NONE, MDTHERMO_ANDERSEN, MDTHERMO_LOWE_ANDERSEN = 0, 1, 2
REPLICA_PERIODIC_MD = 1  # smpc_replica_desc.flags

ERR_BITS = {1: "solvent cell out of range", 2: "monomer cell out of range",
            4: "Verlet list overflow", 8: "non-finite velocity", 32: "gamma iteration limit",
            64: "FENE bond beyond R0", 128: "collide/bin cell mismatch",
            256: "fixed-point cell sum out of range"}

# Every entry point declared in include/smpc.h.
EXPORTS = ("smpc_create", "smpc_destroy", "smpc_last_error", "smpc_n_cells", "smpc_set_fluid",
           "smpc_get_fluid", "smpc_set_monomers", "smpc_get_monomers", "smpc_set_bonds",
           "smpc_init_md", "smpc_md_substeps", "smpc_stage_andersen", "smpc_mpc_step",
           "smpc_cycles",
           "smpc_temperature", "smpc_epot", "smpc_delrx", "smpc_set_delrx",
           "smpc_cell_counts", "smpc_cell_members", "smpc_set_collision_counter", "smpc_verlet_rebuilds",
           "smpc_error_word", "smpc_synchronize", "smpc_cycles_profiled", "smpc_time_cycles",
           "smpc_init_solvent", "smpc_temperature_all", "smpc_temperature_all_noalloc",
           "smpc_set_monomer_state_all", "smpc_cycles_io",
           "smpc_get_monomer_state_all", "smpc_set_variants", "smpc_get_variants",
           "smpc_set_pmd_variant", "smpc_get_pmd_variant",
           "smpc_autotune", "smpc_mpc_bin", "smpc_mpc_collide", "smpc_set_molecules",
           "smpc_molecule_observables_all", "smpc_velocity_profile", "smpc_checkpoint_size",
           "smpc_checkpoint_save", "smpc_checkpoint_load", "smpc_checkpoint_write",
           "smpc_checkpoint_read", "smpc_fourier_modes", "smpc_vacf_start", "smpc_vacf_sample",
           "smpc_vacf_result", "smpc_pressure_tensor_all")

PHASES = ("md_substeps", "cycle_begin", "mono_prep", "fluid_bin", "scan", "build_perm",
          "collide", "cycle_end")


OBS_PER_REP = 16


def profile_bins(L, width):
    """Bins k = floor(p / width) for p in [-L/2, L/2]: floor(L/2w) - floor(-L/2w) + 1."""
    import math
    return int(math.floor(L / (2.0 * width)) - math.floor(-L / (2.0 * width)) + 1)


class SmpcError(RuntimeError):
    pass


class ReplicaDesc(C.Structure):
    _fields_ = [("L", C.c_int * 3), ("n_fluid", C.c_int), ("n_mono", C.c_int),
                ("mol0_size", C.c_int), ("kT", C.c_double), ("shear", C.c_double),
                ("h", C.c_double), ("md_dt", C.c_double), ("lambda_", C.c_double),
                ("r_cut", C.c_double), ("r_verlet", C.c_double), ("solvent_mass", C.c_double),
                ("seed", C.c_uint64), ("potential", C.c_int), ("flags", C.c_int)]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("rng", C.c_int), ("mono_bin", C.c_int),
                ("delrx_mode", C.c_int), ("step_update", C.c_int), ("max_neighbors", C.c_int),
                ("strict_cells", C.c_int), ("device", C.c_int), ("angular_momentum", C.c_int),
                ("md_thermostat", C.c_int), ("andersen_nu", C.c_double),
                ("lowe_radius", C.c_double)]


class Inject(C.Structure):
    _fields_ = [("shift", C.c_void_p), ("gamma", C.c_void_p), ("u_phi", C.c_void_p),
                ("u_theta", C.c_void_p)]


_lib = None


def load(path: Optional[str] = None):
    """Loads libsmpc.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise SmpcError(f"{path} is missing: run starpolymersmd_gb300.build.build() "
                        "(the CUDA library is required; there is no CPU fallback)")
    lib = C.CDLL(path)
    P, I, D = C.c_void_p, C.c_int, C.c_double
    sig = {
        "smpc_create": ([C.POINTER(ReplicaDesc), I, C.POINTER(Options), C.POINTER(P)], I),
        "smpc_destroy": ([P], None),
        "smpc_last_error": ([P], C.c_char_p),
        "smpc_n_cells": ([P, I], I),
        "smpc_set_fluid": ([P, I, P, P], I),
        "smpc_get_fluid": ([P, I, P, P], I),
        "smpc_set_monomers": ([P, I, P, P, P, P, P, P], I),
        "smpc_get_monomers": ([P, I, P, P, P], I),
        "smpc_set_bonds": ([P, I, I, P, P], I),
        "smpc_init_md": ([P], I),
        "smpc_md_substeps": ([P, I, I], I),
        "smpc_cycles_io": ([P, I, P, P, P, P, P], I),
        "smpc_stage_andersen": ([P, I, I, P, P, P], I),
        "smpc_mpc_step": ([P, C.c_long, D, C.POINTER(Inject)], I),
        "smpc_cycles": ([P, I], I),
        "smpc_temperature": ([P, I, C.POINTER(D)], I),
        "smpc_epot": ([P, I, C.POINTER(D)], I),
        "smpc_delrx": ([P, I, C.POINTER(D)], I),
        "smpc_set_delrx": ([P, I, D], I),
        "smpc_cell_counts": ([P, I, P, P], I),
        "smpc_cell_members": ([P, I, P, P], I),
        "smpc_set_collision_counter": ([P, C.c_uint64], I),
        "smpc_verlet_rebuilds": ([P, I, C.POINTER(I)], I),
        "smpc_error_word": ([P, C.POINTER(C.c_uint), P], I),
        "smpc_synchronize": ([P], I),
        "smpc_cycles_profiled": ([P, I, P, I, C.POINTER(D)], I),
        "smpc_time_cycles": ([P, I, C.POINTER(D)], I),
        "smpc_init_solvent": ([P, I, C.c_uint64, I], I),
        "smpc_temperature_all": ([P, P], I),
        "smpc_temperature_all_noalloc": ([P, P], I),
        "smpc_set_monomer_state_all": ([P, P, P], I),
        "smpc_get_monomer_state_all": ([P, P, P, P], I),
        "smpc_set_variants": ([P, I, I, I], I),
        "smpc_get_variants": ([P, C.POINTER(I), C.POINTER(I), C.POINTER(I)], I),
        "smpc_set_pmd_variant": ([P, I], I),
        "smpc_get_pmd_variant": ([P, C.POINTER(I)], I),
        "smpc_autotune": ([P, I, C.c_char_p, I], I),
        "smpc_mpc_bin": ([P, C.c_long, D, P, C.POINTER(I)], I),
        "smpc_mpc_collide": ([P, C.POINTER(Inject)], I),
        "smpc_set_molecules": ([P, I, I, P], I),
        "smpc_molecule_observables_all": ([P, P], I),
        "smpc_velocity_profile": ([P, I, D, P, I, P, I], I),
        "smpc_checkpoint_size": ([P, C.POINTER(C.c_uint64)], I),
        "smpc_checkpoint_save": ([P, P, C.c_uint64], I),
        "smpc_checkpoint_load": ([P, P, C.c_uint64], I),
        "smpc_checkpoint_write": ([P, C.c_char_p], I),
        "smpc_checkpoint_read": ([P, C.c_char_p], I),
        "smpc_fourier_modes": ([P, I, D, P], I),
        "smpc_vacf_start": ([P, I, I, I], I),
        "smpc_vacf_sample": ([P], I),
        "smpc_vacf_result": ([P, P, C.POINTER(C.c_uint64)], I),
        "smpc_pressure_tensor_all": ([P, P], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


class Context:
    """One libsmpc context: one or more independent boxes on one GPU."""

    def __init__(self, replicas: Sequence[dict], precision=FP64, rng=RNG_INJECT,
                 mono_bin=MONOBIN_REFERENCE, delrx_mode=DELRX_REFERENCE, step_update=1,
                 max_neighbors=0, strict_cells=None, device=0, angular_momentum=False,
                 md_thermostat=MDTHERMO_NONE, andersen_nu=0.0, lowe_radius=0.0):
        self.lib = load()
        n = len(replicas)
        descs = (ReplicaDesc * n)()
        self.replicas = []
        for k, r in enumerate(replicas):
            d = descs[k]
            for a in range(3):
                d.L[a] = int(r["L"][a])
            d.n_fluid = int(r["n_fluid"])
            d.n_mono = int(r.get("n_mono", 0))
            d.mol0_size = int(r.get("mol0_size", d.n_mono))
            d.kT = float(r.get("kT", 1.0))
            d.shear = float(r.get("shear", 0.0))
            d.h = float(r.get("h", 0.1))
            d.md_dt = float(r.get("md_dt", 0.01))
            d.lambda_ = float(r.get("lambda", 1.0))
            d.r_cut = float(r.get("r_cut", 1.5))
            d.r_verlet = float(r.get("r_verlet", 2.0))
            d.solvent_mass = float(r.get("solvent_mass", 1.0))
            d.seed = int(r.get("seed", 1))
            d.potential = int(r.get("potential", POT_REF4824))
            d.flags = int(r.get("flags", 0))
            self.replicas.append(dict(r))
        opt = Options(precision, rng, mono_bin, delrx_mode, step_update, max_neighbors,
                      int(precision == FP64 if strict_cells is None else strict_cells), device,
                      int(bool(angular_momentum)), int(md_thermostat), float(andersen_nu),
                      float(lowe_radius))
        h = C.c_void_p()
        rc = self.lib.smpc_create(descs, n, C.byref(opt), C.byref(h))
        if rc != 0:
            raise SmpcError(f"smpc_create failed with code {rc}")
        self.h = h
        self.n_rep = n
        self.precision = precision
        self.step_update = step_update
        self.n_cells = [self.lib.smpc_n_cells(self.h, k) for k in range(n)]
        self._keep = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.smpc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc, what):
        if rc != 0:
            msg = self.lib.smpc_last_error(self.h)
            raise SmpcError(f"{what}: code {rc}: {msg.decode() if msg else ''}")

    # state -------------------------------------------------------------------
    def set_fluid(self, rep, pos, vel):
        n = self.replicas[rep]["n_fluid"]
        self._check(self.lib.smpc_set_fluid(self.h, rep, _p(_f64(pos, (n, 3))),
                                            _p(_f64(vel, (n, 3)))), "set_fluid")

    def get_fluid(self, rep=0):
        n = self.replicas[rep]["n_fluid"]
        pos = np.zeros((n, 3))
        vel = np.zeros((n, 3))
        self._check(self.lib.smpc_get_fluid(self.h, rep, _p(pos), _p(vel)), "get_fluid")
        return pos, vel

    def set_monomers(self, rep, pos, vel, force=None, mass=None, amphi=None, anchor=None):
        n = self.replicas[rep].get("n_mono", 0)
        f = None if force is None else _f64(force, (n, 3))
        m = None if mass is None else _f64(mass, (n,))
        a = None if amphi is None else np.ascontiguousarray(amphi, dtype=np.int32)
        c = None if anchor is None else np.ascontiguousarray(anchor, dtype=np.int32)
        self._check(self.lib.smpc_set_monomers(self.h, rep, _p(_f64(pos, (n, 3))),
                                               _p(_f64(vel, (n, 3))), _p(f), _p(m), _p(a), _p(c)),
                    "set_monomers")

    def get_monomers(self, rep=0):
        n = self.replicas[rep].get("n_mono", 0)
        pos, vel, f = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        self._check(self.lib.smpc_get_monomers(self.h, rep, _p(pos), _p(vel), _p(f)),
                    "get_monomers")
        return pos, vel, f

    def set_bonds(self, rep, src, dst):
        s = np.ascontiguousarray(src, dtype=np.int32)
        d = np.ascontiguousarray(dst, dtype=np.int32)
        self._check(self.lib.smpc_set_bonds(self.h, rep, len(s), _p(s), _p(d)), "set_bonds")

    def init_md(self):
        self._check(self.lib.smpc_init_md(self.h), "init_md")

    # stepping ------------------------------------------------------------------
    def md_substeps(self, n=1, calc_epot=False):
        self._check(self.lib.smpc_md_substeps(self.h, n, int(calc_epot)), "md_substeps")

    def stage_andersen(self, rep, step_start, mono, vel):
        """Andersen resets of the next ``len(step_start) - 1`` substeps from the
        host (replica-local monomer ``mono[e]`` gets ``vel[e]`` in substep s for
        e in [step_start[s], step_start[s + 1])), in place of device draws."""
        st = np.ascontiguousarray(step_start, dtype=np.int32)
        mo = np.ascontiguousarray(mono, dtype=np.int32)
        ve = _f64(np.asarray(vel, dtype=np.float64).reshape(-1, 3))
        self._check(self.lib.smpc_stage_andersen(self.h, rep, len(st) - 1, _p(st), _p(mo),
                                                 _p(ve)), "stage_andersen")

    def mpc_step(self, t, dt, shift=None, gamma=None, u_phi=None, u_theta=None):
        inj = None
        if shift is not None:
            arrs = [_f64(shift).ravel(), _f64(gamma).ravel(), _f64(u_phi).ravel(),
                    _f64(u_theta).ravel()]
            self._keep = arrs
            inj = Inject(*[a.ctypes.data for a in arrs])
        self._check(self.lib.smpc_mpc_step(self.h, t, dt, None if inj is None else C.byref(inj)),
                    "mpc_step")

    def mpc_bin(self, t, dt, shift=None):
        """First phase of MPC::step; returns True when this call binned a collision."""
        arr = None if shift is None else _f64(shift).ravel()
        self._keep_bin = arr
        now = C.c_int()
        self._check(self.lib.smpc_mpc_bin(self.h, t, dt, _p(arr), C.byref(now)), "mpc_bin")
        return bool(now.value)

    def mpc_collide(self, gamma=None, u_phi=None, u_theta=None):
        inj = None
        if gamma is not None:
            arrs = [_f64(gamma).ravel(), _f64(u_phi).ravel(), _f64(u_theta).ravel()]
            self._keep = arrs
            inj = Inject(None, *[a.ctypes.data for a in arrs])
        self._check(self.lib.smpc_mpc_collide(self.h, None if inj is None else C.byref(inj)),
                    "mpc_collide")

    def cycles(self, n):
        self._check(self.lib.smpc_cycles(self.h, n), "cycles")

    def cycles_profiled(self, n):
        """Per-phase device time (ms, summed over n cycles) and total ms."""
        ph = np.zeros(len(PHASES))
        tot = C.c_double()
        self._check(self.lib.smpc_cycles_profiled(self.h, n, _p(ph), len(PHASES), C.byref(tot)),
                    "cycles_profiled")
        return dict(zip(PHASES, ph)), tot.value

    def set_variants(self, bin, collide, md):
        self._check(self.lib.smpc_set_variants(self.h, bin, collide, md), "set_variants")

    def get_variants(self):
        b, c, m = C.c_int(), C.c_int(), C.c_int()
        self._check(self.lib.smpc_get_variants(self.h, C.byref(b), C.byref(c), C.byref(m)),
                    "get_variants")
        return b.value, c.value, m.value

    def set_pmd_variant(self, pmd):
        self._check(self.lib.smpc_set_pmd_variant(self.h, pmd), "set_pmd_variant")

    def get_pmd_variant(self):
        v = C.c_int()
        self._check(self.lib.smpc_get_pmd_variant(self.h, C.byref(v)), "get_pmd_variant")
        return v.value

    def autotune(self, cycles=3):
        """Times each kernel's launch-shape variants on the live workload and
        keeps the fastest; returns the report."""
        import json
        buf = C.create_string_buffer(8192)
        self._check(self.lib.smpc_autotune(self.h, cycles, buf, 8192), "autotune")
        return json.loads(buf.value.decode() or "{}")

    def time_cycles(self, n):
        tot = C.c_double()
        self._check(self.lib.smpc_time_cycles(self.h, n, C.byref(tot)), "time_cycles")
        return tot.value

    def init_solvent(self, rep, seed, reference_velocities=False, shear_profile=False):
        flags = (1 if reference_velocities else 0) | (2 if shear_profile else 0)
        self._check(self.lib.smpc_init_solvent(self.h, rep, seed, flags), "init_solvent")

    def synchronize(self):
        self._check(self.lib.smpc_synchronize(self.h), "synchronize")

    # observables ---------------------------------------------------------------
    def temperature(self, rep=0):
        out = C.c_double()
        self._check(self.lib.smpc_temperature(self.h, rep, C.byref(out)), "temperature")
        return out.value

    def temperature_all(self, out=None):
        out = np.zeros(self.n_rep) if out is None else out
        self._check(self.lib.smpc_temperature_all(self.h, _p(out)), "temperature_all")
        return out

    def set_monomer_state_all(self, pos, vel):
        self._check(self.lib.smpc_set_monomer_state_all(self.h, _p(pos), _p(vel)),
                    "set_monomer_state_all")

    def cycles_io(self, n, pos_in=None, vel_in=None, pos_out=None, vel_out=None, obs_out=None):
        """Monomer state in, n fused cycles, monomer state and observables out,
        with one synchronisation (smpc_cycles_io)."""
        self._check(self.lib.smpc_cycles_io(self.h, n, _p(pos_in), _p(vel_in), _p(pos_out),
                                            _p(vel_out), _p(obs_out)), "cycles_io")

    def get_monomer_state_all(self, pos, vel, force=None):
        self._check(self.lib.smpc_get_monomer_state_all(self.h, _p(pos), _p(vel), _p(force)),
                    "get_monomer_state_all")

    def epot(self, rep=0):
        out = C.c_double()
        self._check(self.lib.smpc_epot(self.h, rep, C.byref(out)), "epot")
        return out.value

    def delrx(self, rep=0):
        out = C.c_double()
        self._check(self.lib.smpc_delrx(self.h, rep, C.byref(out)), "delrx")
        return out.value

    def set_delrx(self, rep, d):
        self._check(self.lib.smpc_set_delrx(self.h, rep, d), "set_delrx")

    def cell_counts(self, rep=0):
        n = self.n_cells[rep]
        tot = np.zeros(n, dtype=np.uint32)
        fl = np.zeros(n, dtype=np.uint32)
        self._check(self.lib.smpc_cell_counts(self.h, rep, _p(tot), _p(fl)), "cell_counts")
        return tot, fl

    def set_molecules(self, rep, mol_start):
        ms = np.ascontiguousarray(mol_start, dtype=np.int32)
        self._check(self.lib.smpc_set_molecules(self.h, rep, len(ms) - 1, _p(ms)), "set_molecules")

    def molecule_observables_all(self):
        """Per replica: R_g, G (3x3), rotation frequency, kinetic energy, temperature, molecules."""
        out = np.zeros((self.n_rep, OBS_PER_REP))
        self._check(self.lib.smpc_molecule_observables_all(self.h, _p(out)),
                    "molecule_observables_all")
        return out

    def velocity_profile(self, rep, width):
        """VelocityX sums (v_x, v_y, count) per bin along x and along y."""
        L = self.replicas[rep]["L"]
        nx, ny = profile_bins(int(L[0]), width), profile_bins(int(L[1]), width)
        xo, yo = np.zeros((nx, 3)), np.zeros((ny, 3))
        self._check(self.lib.smpc_velocity_profile(self.h, rep, width, _p(xo), nx, _p(yo), ny),
                    "velocity_profile")
        return xo, yo

    def cell_members(self, rep=0):
        """(cell of every solvent particle by id, cell of every monomer) at the last sort."""
        fc = np.zeros(self.replicas[rep]["n_fluid"], dtype=np.int32)
        mc = np.zeros(self.replicas[rep].get("n_mono", 0), dtype=np.int32)
        self._check(self.lib.smpc_cell_members(self.h, rep, _p(fc), _p(mc)), "cell_members")
        return fc, mc

    def fourier_modes(self, rep, box_length):
        """The three transverse solvent modes of Fourier_Autocorr (complex, 3 x 3:
        mode along x, y, z by velocity component)."""
        out = np.zeros(18)
        self._check(self.lib.smpc_fourier_modes(self.h, rep, float(box_length), _p(out)),
                    "fourier_modes")
        return (out[0::2] + 1j * out[1::2]).reshape(3, 3)

    def pressure_tensor_all(self):
        """(kinetic, virial): (n_rep, 6) each, components xx yy zz xy xz yz."""
        out = np.zeros((self.n_rep, 12))
        self._check(self.lib.smpc_pressure_tensor_all(self.h, _p(out)), "pressure_tensor_all")
        return out[:, :6], out[:, 6:]

    def vacf_start(self, rep, n_particles, entries):
        self._vacf_entries = int(entries)
        self._check(self.lib.smpc_vacf_start(self.h, rep, int(n_particles), int(entries)),
                    "vacf_start")

    def vacf_sample(self):
        self._check(self.lib.smpc_vacf_sample(self.h), "vacf_sample")

    def vacf_result(self):
        """(lag sums over particles and calculations, number of calculations)."""
        out = np.zeros(self._vacf_entries)
        n = C.c_uint64()
        self._check(self.lib.smpc_vacf_result(self.h, _p(out), C.byref(n)), "vacf_result")
        return out, n.value

    def checkpoint(self) -> bytes:
        """The context's full state (smpc_checkpoint_save)."""
        n = C.c_uint64()
        self._check(self.lib.smpc_checkpoint_size(self.h, C.byref(n)), "checkpoint_size")
        buf = np.empty(n.value, dtype=np.uint8)
        self._check(self.lib.smpc_checkpoint_save(self.h, _p(buf), n.value), "checkpoint_save")
        return buf.tobytes()

    def restore(self, blob: bytes):
        buf = np.frombuffer(blob, dtype=np.uint8)
        self._check(self.lib.smpc_checkpoint_load(self.h, _p(buf), len(buf)), "checkpoint_load")

    def checkpoint_write(self, path: str):
        self._check(self.lib.smpc_checkpoint_write(self.h, os.fsencode(path)), "checkpoint_write")

    def checkpoint_read(self, path: str):
        self._check(self.lib.smpc_checkpoint_read(self.h, os.fsencode(path)), "checkpoint_read")

    def set_collision_counter(self, c):
        self._check(self.lib.smpc_set_collision_counter(self.h, c), "set_collision_counter")

    def verlet_rebuilds(self, rep=0):
        out = C.c_int()
        self._check(self.lib.smpc_verlet_rebuilds(self.h, rep, C.byref(out)), "verlet_rebuilds")
        return out.value

    def error_word(self):
        w = C.c_uint()
        info = np.zeros(3, dtype=np.uint32)
        self._check(self.lib.smpc_error_word(self.h, C.byref(w), _p(info)), "error_word")
        return w.value, info

    def raise_on_device_error(self):
        w, info = self.error_word()
        if w:
            names = [v for b, v in ERR_BITS.items() if w & b]
            raise SmpcError(f"device error word 0x{w:x} ({', '.join(names)}), info {list(info)}")
