"""Scene builders shared by the GPU parity tests (CPU-side only)."""
from __future__ import annotations

import numpy as np


def dam_scene_text(n_side=16, jitter=0.05, box=(0.8, 0.5, 0.5), seed=0,
                   begin=0.055, kernel=0.02, interval=0.5, mass=0.001):
    step = kernel * interval
    end = begin + n_side * step - step * 0.5
    return f'''{{"fluid_block": [{{"begin_x": {begin}, "begin_y": {begin}, "begin_z": {begin},
        "end_x": {end}, "end_y": {end}, "end_z": {end}}}],
        "mass": {mass}, "interval": {interval}, "kernel": {kernel},
        "gas_constant": 57142.857, "rest_density": 1000.0, "viscosity": 0.8,
        "time_step": 0.0001, "gravity_y": -9.81, "jitter": {jitter}, "seed": {seed},
        "xx": {box[0]}, "yy": {box[1]}, "zz": {box[2]}}}'''


def dam_scene(gsph, **kw):
    s = gsph.parse_scene(dam_scene_text(**kw))
    p = gsph.params_init(s)
    return s, p, gsph.lattice(s, p)


def dense_scene(gsph, n_side=40, jitter=0.02, seed=5):
    """The reference default scene's physics (h = 0.03, spacing 0.15 h, about
    300 particles per cell): every cell takes the SMS path."""
    kernel, interval = 0.03, 0.15
    step = np.float32(kernel) * np.float32(interval)
    begin = 0.061
    end = begin + n_side * float(step) - float(step) * 0.5
    text = f'''{{"fluid_block": [{{"begin_x": {begin}, "begin_y": {begin}, "begin_z": {begin},
        "end_x": {end}, "end_y": {end}, "end_z": {end}}}],
        "mass": 0.00027, "interval": {interval}, "jitter": {jitter}, "seed": {seed},
        "xx": 0.6, "yy": 0.5, "zz": 0.5}}'''
    s = gsph.parse_scene(text)
    p = gsph.params_init(s)
    return s, p, gsph.lattice(s, p)


def shuffled(pos, seed=11):
    rng = np.random.default_rng(seed)
    return pos[rng.permutation(len(pos))].copy()


def rel_err(a, b, floor):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)
