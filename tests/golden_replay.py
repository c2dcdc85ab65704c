"""Replays a golden fixture (recorded from the reference) through a stepper.

Used by the CPU tests (C restatement oracle) and the GPU tests (CUDA path):
both consume the same initial state and the same injected draws.
"""
import numpy as np


def load(path):
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def has_star(fx):
    return "mono_pos0" in fx


def collision_index(fx):
    return {int(t): k for k, t in enumerate(fx["coll_steps"])}


def is_andersen(fx):
    """MPC-off fixture driven by the reference's AndersenStochastic."""
    return "andersen_nu" in fx


def andersen_resets(fx, t):
    """(monomer indices, velocities) the reference's draws reset in loop step t."""
    a, b = int(fx["andersen_start"][t]), int(fx["andersen_start"][t + 1])
    return fx["andersen_idx"][a:b], fx["andersen_vel"][a:b]
