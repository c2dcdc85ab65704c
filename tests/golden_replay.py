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
