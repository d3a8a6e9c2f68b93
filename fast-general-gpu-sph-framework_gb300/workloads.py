"""Seeded synthetic scenes for the single-scene, batched and served workloads.

Every scene is a dam-break column on a cubic lattice (dx = 0.01 m, h = 2dx,
jitter +-0.05dx from SplitMix64) with the 262k dam break's physics (Tait EOS
rho0 = 1000, c0 = 20 m/s, viscosity 0.8, dt = 1e-4 s, g = -9.81). The column
sits in the lower-left corner of a box 4x its width long and 2x its height
and depth (the 262,144-particle scene's proportions).
"""
from __future__ import annotations

import math

import numpy as np

DX = 0.01
BEGIN = 0.055   # first lattice plane: just outside the walls' penalty zone


def column_scene_text(nx: int, ny: int, nz: int, seed: int) -> str:
    """Scene JSON of an nx x ny x nz column (x length, y height, z depth)."""
    ends = [BEGIN + n * DX - DX / 2 for n in (nx, ny, nz)]
    box = [4 * nx * DX, 2 * ny * DX, 2 * nz * DX]
    box = [max(b, BEGIN + n * DX + 0.06) for b, n in zip(box, (nx, ny, nz))]
    return f'''{{"fluid_block": [{{"begin_x": {BEGIN}, "begin_y": {BEGIN}, "begin_z": {BEGIN},
        "end_x": {ends[0]:.6f}, "end_y": {ends[1]:.6f}, "end_z": {ends[2]:.6f}}}],
        "mass": 0.001, "interval": 0.5, "kernel": 0.02, "rest_density": 1000.0,
        "gas_constant": 57142.857, "viscosity": 0.8, "time_step": 0.0001,
        "gravity_y": -9.81, "jitter": 0.05, "seed": {seed},
        "xx": {box[0]:.6f}, "yy": {box[1]:.6f}, "zz": {box[2]:.6f}}}'''


def column_shape(n_target: float, aspect: float):
    """Column dimensions with about n_target particles, height = aspect x width."""
    w = max(2, int(round((n_target / aspect) ** (1.0 / 3.0))))
    hgt = max(2, int(round(aspect * w)))
    return w, hgt, w


def batched_scenes(num_scenes: int = 256, seed: int = 0, n_min: int = 4096,
                   n_max: int = 262144):
    """Scene specs of the batched workload: N log-uniform in [n_min, n_max],
    column aspect (height / width) uniform in [0.5, 2]; scene i uses seed i."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(num_scenes):
        n = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        a = rng.uniform(0.5, 2.0)
        nx, ny, nz = column_shape(n, a)
        specs.append({"nx": nx, "ny": ny, "nz": nz, "seed": seed * 100003 + i,
                      "aspect": a})
    return specs


def build(g, spec):
    """(params, positions) of one scene spec via the library's host code."""
    s = g.parse_scene(column_scene_text(spec["nx"], spec["ny"], spec["nz"], spec["seed"]))
    p = g.params_init(s)
    return p, g.lattice(s, p)


def served_requests(duration_s: float = 60.0, rate_hz: float = 50.0, seed: int = 1,
                    n_min: int = 8192, n_max: int = 1048576, k_min: int = 50,
                    k_max: int = 500):
    """Poisson arrivals: (arrival time, scene spec, steps) for the served
    workload (N log-uniform in [n_min, n_max], K uniform in [k_min, k_max])."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    i = 0
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= duration_s:
            break
        n = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        a = rng.uniform(0.5, 2.0)
        nx, ny, nz = column_shape(n, a)
        k = int(rng.integers(k_min, k_max + 1))
        out.append((t, {"nx": nx, "ny": ny, "nz": nz, "seed": 7_000_000 + i, "aspect": a}, k))
        i += 1
    return out
