"""System construction: star topology, initial conditions and replica tables.

Index layout and bond order follow the reference's star builder
(star-polymers/lib/Molecules/Molecule.cpp:126-176): the core (anchor) is
monomer 0; bead k (1..A+B) of arm a is monomer a*(A+B)+k; beads with k > A are
solvophobic (AmphiType 1); the directed FENE bonds are core -> first bead of
every arm (stored by MDParticle::set_neighbor with push_front, so the core
lists its arms in reverse order, Particle.cpp:38-40) and bead k -> bead k+1.
"""
from __future__ import annotations

import dataclasses
import json
import math
import os
from typing import List, Optional, Sequence

import numpy as np


@dataclasses.dataclass
class Star:
    """Topology and state of one star polymer (reference index layout)."""
    arms: int
    A: int
    B: int
    mass: float
    pos: np.ndarray          # (N, 3)
    vel: np.ndarray          # (N, 3)
    amphi: np.ndarray        # (N,) int32, 1 = solvophobic
    anchor: np.ndarray       # (N,) int32, 1 = core
    bond_src: np.ndarray     # directed bonds (MDParticle::Neighbors order)
    bond_dst: np.ndarray

    @property
    def n(self) -> int:
        return 1 + self.arms * (self.A + self.B)


def star_topology(arms: int, A: int, B: int):
    """Types, anchor flags and directed bonds of a star (Molecule.cpp:126-176)."""
    npa = A + B
    n = 1 + arms * npa
    amphi = np.zeros(n, dtype=np.int32)
    anchor = np.zeros(n, dtype=np.int32)
    anchor[0] = 1
    src, dst = [], []
    # core -> first bead of each arm, pushed to the front: reverse arm order
    for a in reversed(range(arms)):
        src.append(0)
        dst.append(a * npa + 1)
    for a in range(arms):
        for k in range(1, npa + 1):
            idx = a * npa + k
            if k > A:
                amphi[idx] = 1
            if k < npa:
                src.append(idx)
                dst.append(idx + 1)
    # group by source monomer, keeping per-source order (Neighbors lists)
    order = sorted(range(len(src)), key=lambda b: (src[b], b))
    return (amphi, anchor, np.array([src[b] for b in order], dtype=np.int32),
            np.array([dst[b] for b in order], dtype=np.int32))


def saw_star(arms: int, n_arm: int, rng: np.random.Generator, bond: float = 1.0,
             anchor_bond: float = 2.0, r_min: float = 1.0, outward_bias: float = 0.5,
             max_tries: int = 400, centre=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Self-avoiding random-walk star grown from ``centre``.

    Arm roots sit ``anchor_bond`` from the core on a Fibonacci sphere (randomly
    rotated); the arms then grow round-robin, one bead per arm per round, each
    step of length ``bond`` in a random direction with an ``outward_bias``
    toward the radial direction. A bead is accepted when it is farther than
    ``r_min`` from every bead placed so far except its bonded predecessor.
    Bead order in the result is the reference's star layout: core, then arm
    by arm from the core outward.
    """
    c = np.asarray(centre, dtype=np.float64)
    n = 1 + arms * n_arm
    placed = np.zeros((n, 3))
    placed[0] = c
    count = 1
    arm_beads = [[] for _ in range(arms)]
    # roots on a randomly rotated Fibonacci sphere
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    golden = math.pi * (3.0 - math.sqrt(5.0))
    for a in range(arms):
        z = 1.0 - 2.0 * (a + 0.5) / arms
        r = math.sqrt(max(0.0, 1.0 - z * z))
        d = q @ np.array([r * math.cos(golden * a), r * math.sin(golden * a), z])
        p = c + d * anchor_bond
        placed[count] = p
        count += 1
        arm_beads[a].append(p)

    def free(x, skip):
        dd = placed[:count] - x
        ok = np.einsum("ij,ij->i", dd, dd) > r_min * r_min
        ok[skip] = True  # the bonded predecessor sits at the bond length
        return bool(np.all(ok))

    last_index = list(range(1, arms + 1))
    for _k in range(1, n_arm):
        for a in range(arms):
            prev = arm_beads[a][-1]
            radial = prev - c
            radial /= max(np.linalg.norm(radial), 1e-12)
            for _t in range(max_tries):
                s = rng.normal(size=3)
                s /= np.linalg.norm(s)
                s = s + outward_bias * radial
                s /= np.linalg.norm(s)
                x = prev + s * bond
                if free(x, last_index[a]):
                    break
            else:
                raise RuntimeError("self-avoiding walk got stuck")
            placed[count] = x
            last_index[a] = count
            count += 1
            arm_beads[a].append(x)
    out = np.zeros((n, 3))
    out[0] = c
    for a in range(arms):
        out[1 + a * n_arm: 1 + (a + 1) * n_arm] = np.asarray(arm_beads[a])
    return out


def thermal_velocities(n: int, mass: float, kT: float, rng: np.random.Generator) -> np.ndarray:
    """Maxwell-Boltzmann velocities with zero mean."""
    v = rng.normal(scale=math.sqrt(kT / mass), size=(n, 3))
    v -= v.mean(axis=0)
    return v


def make_star(arms: int, n_arm: int, solvophobic_fraction: float, mass: float, kT: float,
              rng: np.random.Generator, bond: float = 1.0, anchor_bond: float = 2.0,
              r_min: float = 1.0, centre=(0.0, 0.0, 0.0), outward_bias: float = 0.5) -> Star:
    B = int(round(solvophobic_fraction * n_arm))
    A = n_arm - B
    amphi, anch, src, dst = star_topology(arms, A, B)
    pos = saw_star(arms, n_arm, rng, bond=bond, anchor_bond=anchor_bond, r_min=r_min,
                   centre=centre, outward_bias=outward_bias)
    vel = thermal_velocities(len(pos), mass, kT, rng)
    return Star(arms, A, B, mass, pos, vel, amphi, anch, src, dst)


def uniform_fluid(L: Sequence[int], n_c: int, kT: float, rng: np.random.Generator,
                  reference_velocities: bool = False):
    """Solvent at n_c particles per cell: positions uniform in the box.

    Velocities are Maxwell-Boltzmann at kT, or with ``reference_velocities``
    uniform in [-1/2, 1/2) minus their mean as MPC::initialize does
    (MPC.cpp:34-55).
    """
    n = int(n_c * L[0] * L[1] * L[2])
    pos = (rng.random((n, 3)) - 0.5) * np.asarray(L, dtype=np.float64)
    if reference_velocities:
        vel = rng.random((n, 3)) - 0.5
        vel -= vel.mean(axis=0)
    else:
        vel = thermal_velocities(n, 1.0, kT, rng)
    return pos, vel


@dataclasses.dataclass
class ReplicaSpec:
    """Parameters of one independent system (one box, its stars, its solvent)."""
    L: int
    arms: int
    n_arm: int
    solvophobic_fraction: float
    shear: float
    seed: int
    n_c: int = 10
    mono_mass: float = 5.0
    kT: float = 1.0
    n_stars: int = 1


def batched_replica_table(n: int = 256, seed: int = 1) -> List[ReplicaSpec]:
    """Uneven replica set: f ~ U{3..12}, N_arm ~ U{10..60}, solvophobic fraction
    ~ U[0.2, 0.8], cubic L ~ U{16..40}, shear log-uniform in [1e-3, 0.5],
    distinct seeds 1..n; drawn from numpy's default generator seeded with 1."""
    rng = np.random.default_rng(seed)
    f = rng.integers(3, 13, size=n)
    na = rng.integers(10, 61, size=n)
    frac = rng.uniform(0.2, 0.8, size=n)
    L = rng.integers(16, 41, size=n)
    shear = np.exp(rng.uniform(math.log(1e-3), math.log(0.5), size=n))
    return [ReplicaSpec(L=int(L[i]), arms=int(f[i]), n_arm=int(na[i]),
                        solvophobic_fraction=float(frac[i]), shear=float(shear[i]),
                        seed=i + 1) for i in range(n)]


def replica_table_json(specs: Sequence[ReplicaSpec]) -> str:
    return json.dumps([dataclasses.asdict(s) for s in specs], indent=0)


@dataclasses.dataclass
class StarSolution:
    """Several stars in one periodic box, concatenated star by star (each in
    the reference's star layout); positions are unwrapped (every star
    contiguous) and may reach outside the primary box."""
    stars: List[Star]
    L: tuple

    @property
    def n(self) -> int:
        return sum(s.n for s in self.stars)

    @property
    def mol_start(self) -> np.ndarray:
        return np.concatenate([[0], np.cumsum([s.n for s in self.stars])]).astype(np.int32)

    def _cat(self, name):
        return np.concatenate([getattr(s, name) for s in self.stars])

    @property
    def pos(self) -> np.ndarray:
        return self._cat("pos")

    @property
    def vel(self) -> np.ndarray:
        return self._cat("vel")

    @property
    def amphi(self) -> np.ndarray:
        return self._cat("amphi")

    @property
    def anchor(self) -> np.ndarray:
        return self._cat("anchor")

    @property
    def mass(self) -> np.ndarray:
        return np.concatenate([np.full(s.n, s.mass) for s in self.stars])

    @property
    def bond_src(self) -> np.ndarray:
        off = self.mol_start
        return np.concatenate([s.bond_src + off[k] for k, s in enumerate(self.stars)]).astype(np.int32)

    @property
    def bond_dst(self) -> np.ndarray:
        off = self.mol_start
        return np.concatenate([s.bond_dst + off[k] for k, s in enumerate(self.stars)]).astype(np.int32)


class _PeriodicOccupancy:
    """Placed beads of a periodic box on a hash grid of unit cells, for
    self-avoidance checks under the minimum image (no shear offset: set-up
    happens at delrx = 0)."""

    def __init__(self, L, cell: float = 1.0):
        self.L = np.asarray(L, dtype=np.float64)
        self.n = np.maximum(1, np.floor(self.L / cell)).astype(int)
        self.side = self.L / self.n
        self.cells = {}

    def _key(self, x):
        return tuple((np.floor((x + 0.5 * self.L) / self.side).astype(int) % self.n).tolist())

    def add(self, idx: int, x) -> None:
        self.cells.setdefault(self._key(x), []).append((idx, np.array(x, dtype=np.float64)))

    def free(self, x, r_min: float, skip: int = -1) -> bool:
        k = np.array(self._key(x))
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    c = tuple(((k + (dx, dy, dz)) % self.n).tolist())
                    for idx, p in self.cells.get(c, ()):
                        if idx == skip:
                            continue
                        d = p - x
                        d -= self.L * np.round(d / self.L)
                        if float(d @ d) <= r_min * r_min:
                            return False
        return True


def star_solution(n_stars: int, arms: int, n_arm: int, solvophobic_fraction: float,
                  mass: float, kT: float, L: Sequence[int], rng: np.random.Generator,
                  bond: float = 1.0, anchor_bond: float = 2.0, r_min: float = 1.0,
                  outward_bias: float = 0.5, jitter: float = 0.25,
                  max_tries: int = 400) -> StarSolution:
    """``n_stars`` self-avoiding stars (no bead within ``r_min`` of another,
    across stars and periodic images) with their cores on a randomised cubic
    lattice: the first ``n_stars`` sites of a ceil(n^(1/3))-per-axis lattice,
    in random order, each core moved by up to ``jitter`` of the spacing along
    every axis. Arms grow round-robin as in ``saw_star``."""
    Lv = np.asarray(L, dtype=np.float64)
    m = int(math.ceil(n_stars ** (1.0 / 3.0) - 1e-9))
    sites = np.array([(i, j, k) for i in range(m) for j in range(m) for k in range(m)])
    sites = sites[rng.permutation(len(sites))[:n_stars]]
    spacing = Lv / m
    centres = -0.5 * Lv + (sites + 0.5) * spacing
    centres += rng.uniform(-jitter, jitter, size=centres.shape) * spacing
    occ = _PeriodicOccupancy(Lv)
    B = int(round(solvophobic_fraction * n_arm))
    A = n_arm - B
    amphi, anch, src, dst = star_topology(arms, A, B)
    golden = math.pi * (3.0 - math.sqrt(5.0))
    stars = []
    base = 0
    for c in centres:
        n = 1 + arms * n_arm
        for _attempt in range(50):
            q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            roots = []
            for a in range(arms):
                z = 1.0 - 2.0 * (a + 0.5) / arms
                r = math.sqrt(max(0.0, 1.0 - z * z))
                roots.append(c + (q @ np.array([r * math.cos(golden * a),
                                                r * math.sin(golden * a), z])) * anchor_bond)
            if occ.free(c, r_min) and all(occ.free(p, r_min) for p in roots):
                break
        else:
            raise RuntimeError("no free place for a star core")
        occ.add(base, c)
        arm_beads = [[p] for p in roots]
        last = []
        for a, p in enumerate(roots):
            occ.add(base + 1 + a * n_arm, p)
            last.append(base + 1 + a * n_arm)
        for k in range(1, n_arm):
            for a in range(arms):
                prev = arm_beads[a][-1]
                radial = prev - c
                radial /= max(np.linalg.norm(radial), 1e-12)
                for _t in range(max_tries):
                    s = rng.normal(size=3)
                    s /= np.linalg.norm(s)
                    s = s + outward_bias * radial
                    s /= np.linalg.norm(s)
                    x = prev + s * bond
                    if occ.free(x, r_min, skip=last[a]):
                        break
                else:
                    raise RuntimeError("self-avoiding walk got stuck")
                idx = base + 1 + a * n_arm + k
                occ.add(idx, x)
                last[a] = idx
                arm_beads[a].append(x)
        pos = np.zeros((n, 3))
        pos[0] = c
        for a in range(arms):
            pos[1 + a * n_arm: 1 + (a + 1) * n_arm] = np.asarray(arm_beads[a])
        vel = thermal_velocities(n, mass, kT, rng)
        stars.append(Star(arms, A, B, mass, pos, vel, amphi.copy(), anch.copy(), src.copy(),
                          dst.copy()))
        base += n
    return StarSolution(stars, tuple(int(x) for x in L))
