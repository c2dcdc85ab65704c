"""The reference's restart and trajectory text formats, read and written on
the host, so a run can continue from the reference's files and the
reference's tools can read this framework's output.

* fluid: one particle per line, ``x y z vx vy vz`` as ``%f`` with a trailing
  space (MPC::print_fluid_complete, star-polymers/lib/Hydrodynamics/MPC.cpp:570-579),
  read back as MPC::initialize(filename, Box_old) does (MPC.cpp:57-113);
* stars: PDB models with velocities, coordinates and velocities as ``%7.3f``
  at fixed columns, star CONECT records (Box::print_PDB_with_velocity,
  star-polymers/lib/Box.cpp:563-602), read back as Molecule::star_from_file
  does (star-polymers/lib/Molecules/Molecule.cpp:178-224).

Both formats round to a few decimals; for an exact restart use the binary
checkpoint of the C ABI (``Context.checkpoint`` / ``smpc_checkpoint_*``).
"""
from __future__ import annotations

from typing import IO, Iterable, Optional, Sequence, Tuple, Union

import numpy as np

from . import system

PathOrFile = Union[str, IO[str]]


def _open(f: PathOrFile, mode: str):
    if isinstance(f, str):
        return open(f, mode), True
    return f, False


def c_round(x):
    """C's round(): halves away from zero (numpy rounds halves to even)."""
    x = np.asarray(x, dtype=np.float64)
    t = np.trunc(x)
    return t + np.where(np.abs(x - t) >= 0.5, np.sign(x), 0.0)


# ------------------------------------------------------------------ fluid

def write_fluid_complete(f: PathOrFile, pos: np.ndarray, vel: np.ndarray) -> None:
    """MPC::print_fluid_complete: ``%f %f %f %f %f %f \\n`` per particle."""
    fh, own = _open(f, "w")
    try:
        p = np.asarray(pos, dtype=np.float64)
        v = np.asarray(vel, dtype=np.float64)
        fh.writelines("%f %f %f %f %f %f \n" % (a[0], a[1], a[2], b[0], b[1], b[2])
                      for a, b in zip(p, v))
    finally:
        if own:
            fh.close()


def _le_wrap(x: np.ndarray, v: np.ndarray, L: Sequence[int], shear: float, delrx: float) -> None:
    """MPC::wrap(Particle&) in place: LEBC with the velocity jump when the
    shear is on (MPC.cpp:421-429), else the plain periodic wrap (MPC.cpp:487-490)."""
    Lx, Ly, Lz = (float(a) for a in L)
    if shear != 0.0:
        cy = c_round(x[:, 1] / Ly)
        x[:, 0] -= Lx * c_round(x[:, 0] / Lx)
        x[:, 0] -= cy * delrx
        x[:, 0] -= Lx * c_round(x[:, 0] / Lx)
        x[:, 1] -= Ly * cy
        x[:, 2] -= Lz * c_round(x[:, 2] / Lz)
        v[:, 0] -= cy * shear * Ly
    else:
        for d, Ld in enumerate((Lx, Ly, Lz)):
            x[:, d] -= c_round(x[:, d] / Ld) * Ld


def read_fluid(f: PathOrFile, n_fluid: int, L: Sequence[int], L_old: Optional[Sequence[int]] = None,
               shear: float = 0.0, delrx: float = 0.0,
               rng: Optional[np.random.Generator] = None) -> Tuple[np.ndarray, np.ndarray, int, int]:
    """MPC::initialize(filename, Box_old): the first ``n_fluid`` lines give
    particles; a particle whose position lies outside the new box (any
    |round(x_d / L_d)| >= 1), and every particle the file has no line for,
    is placed at random -- in the slab the box grew by when it grew along
    that axis, else anywhere -- with velocity components uniform in
    [-1/2, 1/2). Every particle is wrapped into the box, then the mean
    velocity is removed. Returns (pos, vel, from file, added). The random
    fill draws from ``rng`` (numpy), not from the reference's generator."""
    L = [int(a) for a in L]
    L_old = [int(a) for a in (L_old if L_old is not None else L)]
    rng = rng if rng is not None else np.random.default_rng()
    fh, own = _open(f, "r")
    try:
        vals = []
        for line in fh:
            vals.extend(float(t) for t in line.split())
            if len(vals) >= 6 * n_fluid:
                break
    finally:
        if own:
            fh.close()
    n_file = min(len(vals) // 6, n_fluid)
    data = np.asarray(vals[:6 * n_file], dtype=np.float64).reshape(n_file, 6)
    pos = np.zeros((n_fluid, 3))
    vel = np.zeros((n_fluid, 3))
    Lv = np.asarray(L, dtype=np.float64)
    outside = np.ones(n_fluid, dtype=bool)
    if n_file:
        inside = np.all(np.abs(c_round(data[:, :3] / Lv)) < 1.0, axis=1)
        outside[:n_file] = ~inside
        pos[:n_file][inside] = data[inside, :3]
        vel[:n_file][inside] = data[inside, 3:]
    for i in np.nonzero(outside)[0]:
        for d in range(3):
            r = rng.random()
            grow = L[d] - L_old[d]
            if grow > 0:
                r = -L[d] * 0.5 + grow * r if r < 0.5 else L_old[d] * 0.5 + grow * (r - 0.5)
            else:
                r = L[d] * (r - 0.5)
            pos[i, d] = r
            vel[i, d] = rng.random() - 0.5
    _le_wrap(pos, vel, L, shear, delrx)
    # the mean velocity summed particle by particle, as the reference does
    cmv = np.add.accumulate(vel, axis=0)[-1] / n_fluid if n_fluid else np.zeros(3)
    vel -= cmv
    n_added = int(outside.sum())
    return pos, vel, n_fluid - n_added, n_added


# ------------------------------------------------------------------ stars

def _star_conect(arms: int, per_arm: int) -> Iterable[str]:
    """CONECT records of one star (Box.cpp:578-597): the core's partners five
    to a line, then core-first-bead, bead chains and arm ends."""
    count, arm = 1, 0
    while arm < arms:
        line = "CONECT %4i " % 1
        while count % 5:
            line += "%4i " % (arm * per_arm + 2)
            arm += 1
            count += 1
            if arm >= arms:
                break
        count = 1
        yield line + "\n"
    for i in range(arms):
        yield "CONECT %4u %4u \n" % (i * per_arm + 2, 1)
        for j in range(1, per_arm):
            number = i * per_arm + j
            yield "CONECT %4u %4u %4u \n" % (number + 1, number, number + 2)
        yield "CONECT %4u %4u \n" % ((i + 1) * per_arm + 1, (i + 1) * per_arm)


def write_pdb_with_velocity(f: PathOrFile, step: int, stars: Sequence[system.Star],
                            pos: Optional[np.ndarray] = None,
                            vel: Optional[np.ndarray] = None) -> None:
    """One PDB model of every star (Box::print_PDB_with_velocity): ATOM
    records ``C`` for solvophobic and ``O`` for solvophilic beads with
    position and velocity, TER, the star's CONECT records, ENDMDL. ``pos`` /
    ``vel`` (all stars concatenated) override the stars' own arrays."""
    fh, own = _open(f, "w")
    try:
        fh.write("MODEL     %d \n" % step)
        off = 0
        for m, st in enumerate(stars):
            p = st.pos if pos is None else np.asarray(pos)[off:off + st.n]
            v = st.vel if vel is None else np.asarray(vel)[off:off + st.n]
            for i in range(st.n):
                atom = "C" if st.amphi[i] else "O"
                fh.write("ATOM %6d  %s   GLY    %2d     %7.3f %7.3f %7.3f %7.3f %7.3f %7.3f \n"
                         % (i, atom, m + 1, p[i, 0], p[i, 1], p[i, 2], v[i, 0], v[i, 1], v[i, 2]))
            fh.write("TER \n")
            fh.writelines(_star_conect(st.arms, st.A + st.B))
            off += st.n
        fh.write("ENDMDL \n")
    finally:
        if own:
            fh.close()


def read_star_pdb(f: PathOrFile, arms: int, A: int, B: int, mass: float = 1.0,
                  set_zero: bool = False) -> system.Star:
    """Molecule::star_from_file: skip one line, then read the star's
    1 + arms (A + B) ATOM lines at the fixed columns 31, 39, 47 (position)
    and 55, 63, 71 (velocity), 7 characters each; with ``set_zero`` the
    (unweighted) centre of mass and its velocity are removed. Topology and
    types are the star layout's (system.star_topology)."""
    n = 1 + arms * (A + B)
    fh, own = _open(f, "r")
    try:
        fh.readline()
        rows = [fh.readline() for _ in range(n)]
    finally:
        if own:
            fh.close()
    pos = np.array([[float(r[31:38]), float(r[39:46]), float(r[47:54])] for r in rows])
    vel = np.array([[float(r[55:62]), float(r[63:70]), float(r[71:78])] for r in rows])
    if set_zero:
        pos -= np.add.accumulate(pos, axis=0)[-1] / n
        vel -= np.add.accumulate(vel, axis=0)[-1] / n
    amphi, anchor, src, dst = system.star_topology(arms, A, B)
    return system.Star(arms, A, B, mass, pos, vel, amphi, anchor, src, dst)


def read_pdb_models(f: PathOrFile):
    """Every MODEL of a PDB-with-velocity file (this framework's extension
    for many stars): a list of (step, [(pos, vel) per molecule])."""
    fh, own = _open(f, "r")
    try:
        models, cur, step = [], None, None
        for line in fh:
            if line.startswith("MODEL"):
                step, cur = int(line.split()[1]), {}
            elif line.startswith("ATOM") and cur is not None:
                mol = int(line[24:26])
                p = [float(line[31:38]), float(line[39:46]), float(line[47:54])]
                v = [float(line[55:62]), float(line[63:70]), float(line[71:78])]
                cur.setdefault(mol, []).append(p + v)
            elif line.startswith("ENDMDL") and cur is not None:
                mols = [np.asarray(cur[k]) for k in sorted(cur)]
                models.append((step, [(m[:, :3], m[:, 3:]) for m in mols]))
                cur = None
    finally:
        if own:
            fh.close()
    return models
