"""CPU oracle of the WCSPH step (ctypes wrapper of sph_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker. The product (libgsph.so and its
Python mirror) never imports or calls this module.

`build()` compiles sph_oracle.c with gcc (-O2 -fopenmp) into oracle/lib/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SRC = HERE / "sph_oracle.c"
LIB = HERE / "lib" / "liboracle.so"

_lib = None


def build(force: bool = False) -> Path:
    LIB.parent.mkdir(exist_ok=True)
    deps = [SRC, ROOT / "include" / "gsph.h"]
    if force or not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        cmd = ["gcc", "-std=gnu11", "-O2", "-fopenmp", "-fPIC", "-shared",
               "-ffp-contract=off", "-o", str(LIB), str(SRC), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def _load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        vp = C.c_void_p
        sig = {
            "oracle_params_init": ([vp, vp], C.c_int),
            "oracle_lattice": ([vp, vp, vp, C.c_long], C.c_long),
            "oracle_keys": ([vp, C.c_long, vp, vp], C.c_int),
            "oracle_sort": ([vp, C.c_long, vp, vp, vp, vp], C.c_int),
            "oracle_block_req": ([vp, vp, vp], None),
            "oracle_split": ([vp, vp, vp, vp], C.c_long),
            "oracle_tasks": ([vp, vp, vp, vp, vp, C.c_long], C.c_long),
            "oracle_density": ([vp, vp, vp, C.c_long, vp, vp, vp], C.c_int),
            "oracle_force": ([vp, vp, vp, vp, C.c_long, vp, vp, vp], C.c_int),
            "oracle_force_model": ([vp, vp, vp, vp, C.c_long, vp, C.c_int, C.c_double,
                                    C.c_double, vp, vp], C.c_int),
            "oracle_integrate": ([vp, vp, vp, vp, C.c_long, vp], None),
            "oracle_step": ([vp, vp, vp, C.c_long, vp], C.c_int),
            "oracle_num_threads": ([], C.c_int),
        }
        for name, (args, res) in sig.items():
            fn = getattr(_lib, name)
            fn.argtypes = args
            fn.restype = res
    return _lib


def _p(a):
    return a.ctypes.data


def _ref(struct):
    return C.addressof(struct)


def num_threads() -> int:
    return int(_load().oracle_num_threads())


def scene_from_json(text, scene_cls, max_blocks: int = 64):
    """readSceneFromJsonFile (src/simulation/sph_hybrid_system.cpp:69-126) with
    the Scene defaults of sph_hybrid_system.h:37-44, restated on Python's json
    reader: numbers are read as doubles and stored as floats; a missing
    fluid_block bound reads 0 (jsoncpp's null); the optional physics keys stay
    NaN when absent (parameter defaults apply)."""
    import json
    d = json.loads(text)
    s = scene_cls()
    nan = float("nan")
    s.interval, s.mass, s.recomm_nump = 0.5, 0.02, 65536
    for name in ("kernel", "rest_density", "gas_constant", "viscosity", "time_step",
                 "gravity_y"):
        setattr(s, name, nan)
    s.jitter, s.seed = 0.0, 0
    for a, k in enumerate(("xx", "yy", "zz")):
        if k in d:
            s.world[a] = float(d[k])
    for k in ("mass", "interval", "kernel", "rest_density", "gas_constant", "viscosity",
              "time_step", "gravity_y", "jitter"):
        if k in d:
            setattr(s, k, float(d[k]))
    if "recomm_nump" in d:
        s.recomm_nump = int(d["recomm_nump"])
    if "seed" in d:
        s.seed = int(d["seed"])
    blocks = d.get("fluid_block", [])
    if len(blocks) > max_blocks:
        raise ValueError(f"scene has {len(blocks)} fluid blocks (max {max_blocks})")
    for i, b in enumerate(blocks):
        for a, ax in enumerate("xyz"):
            s.block_begin[i][a] = float(b.get(f"begin_{ax}", 0.0))
            s.block_end[i][a] = float(b.get(f"end_{ax}", 0.0))
    s.n_blocks = len(blocks)
    return s


def params_init(scene, params_cls):
    """defaultInitializeSPHSysPara restated; returns a new params struct."""
    p = params_cls()
    if _load().oracle_params_init(_ref(scene), _ref(p)) != 0:
        raise ValueError("grid size out of range")
    return p


def lattice(scene, params) -> np.ndarray:
    lib = _load()
    n = lib.oracle_lattice(_ref(scene), _ref(params), None, 0)
    out = np.zeros((max(n, 1), 4), np.float32)
    lib.oracle_lattice(_ref(scene), _ref(params), _p(out), n)
    return out[:n].copy()


def numc(params) -> int:
    return int(params.grid_size[0]) * int(params.grid_size[1]) * int(params.grid_size[2])


def keys(pos4: np.ndarray, params) -> np.ndarray:
    pos4 = np.ascontiguousarray(pos4, np.float32)
    out = np.empty(len(pos4), np.uint32)
    _load().oracle_keys(_p(pos4), len(pos4), _ref(params), _p(out))
    return out


def sort(pos4: np.ndarray, params):
    """Canonical grid sort: returns (key_sorted, perm, cell_start, out_of_grid)."""
    pos4 = np.ascontiguousarray(pos4, np.float32)
    n = len(pos4)
    ks = np.empty(n, np.uint32)
    perm = np.empty(n, np.int32)
    cs = np.empty(numc(params) + 1, np.int32)
    bad = _load().oracle_sort(_p(pos4), n, _ref(params), _p(ks), _p(perm), _p(cs))
    if bad < 0:
        raise MemoryError("oracle_sort allocation failed")
    return ks, perm, cs, bool(bad)


def micro_start(key_sorted: np.ndarray, params) -> np.ndarray:
    """Dense micro-cell offsets (numc*64 + 1) of a sorted key array."""
    m = numc(params) * 64
    counts = np.bincount(key_sorted.astype(np.int64), minlength=m)[:m]
    out = np.zeros(m + 1, np.int32)
    np.cumsum(counts, out=out[1:])
    return out


def block_req(cell_start: np.ndarray, params) -> np.ndarray:
    cs = np.ascontiguousarray(cell_start, np.int32)
    out = np.empty(numc(params), np.int32)
    _load().oracle_block_req(_p(cs), _ref(params), _p(out))
    return out


def split(cell_start: np.ndarray, req: np.ndarray, params):
    """Returns (compact index, middle)."""
    cs = np.ascontiguousarray(cell_start, np.int32)
    rq = np.ascontiguousarray(req, np.int32)
    out = np.empty(int(cs[-1]), np.int32)
    middle = _load().oracle_split(_p(cs), _p(rq), _ref(params), _p(out))
    return out, int(middle)


def tasks(key_sorted, cell_start, req, params, task_dtype) -> np.ndarray:
    """SMS task descriptors (knArrangeSmsTasks + judgeTask); T + (T & 1) rows."""
    ks = np.ascontiguousarray(key_sorted, np.uint32)
    cs = np.ascontiguousarray(cell_start, np.int32)
    rq = np.ascontiguousarray(req, np.int32)
    cap = int(rq.sum()) + 2
    out = np.zeros(cap, task_dtype)
    t = _load().oracle_tasks(_p(ks), _p(cs), _p(rq), _ref(params), _p(out), cap)
    if t < 0:
        raise RuntimeError("task capacity exceeded")
    return out[: t + (t & 1)].copy()


def density(pos4_sorted, key_sorted, cell_start, params):
    """Returns (rho, pressure) in float64."""
    p = np.ascontiguousarray(pos4_sorted, np.float32)
    n = len(p)
    rho = np.empty(n, np.float64)
    pr = np.empty(n, np.float64)
    if _load().oracle_density(_p(p), _p(np.ascontiguousarray(key_sorted, np.uint32)),
                              _p(np.ascontiguousarray(cell_start, np.int32)), n,
                              _ref(params), _p(rho), _p(pr)) != 0:
        raise MemoryError("oracle_density allocation failed")
    return rho, pr


def force(pos4_sorted, ev4_sorted, key_sorted, cell_start, params, with_mag=False,
          artificial=None):
    """FP64 force (n, 3); with_mag also returns the per-particle sum of pair
    term magnitudes (the conditioning scale of the summation). artificial =
    (alpha, c0) replaces the reference's Laplacian viscosity with Monaghan's
    artificial viscosity."""
    p = np.ascontiguousarray(pos4_sorted, np.float32)
    e = np.ascontiguousarray(ev4_sorted, np.float32)
    n = len(p)
    acc = np.empty((n, 3), np.float64)
    mag = np.empty(n, np.float64)
    model, alpha, c0 = (0, 0.0, 0.0) if artificial is None else (1, *artificial)
    if _load().oracle_force_model(_p(p), _p(e),
                                  _p(np.ascontiguousarray(key_sorted, np.uint32)),
                                  _p(np.ascontiguousarray(cell_start, np.int32)), n,
                                  _ref(params), model, float(alpha), float(c0),
                                  _p(acc), _p(mag)) != 0:
        raise MemoryError("oracle_force allocation failed")
    return (acc, mag) if with_mag else acc


def integrate(pos4, vel4, ev4, acc3, params):
    """FP64 integrator; returns new (pos4, vel4, ev4) as float64 arrays."""
    p = np.array(pos4, np.float64, order="C")
    v = np.array(vel4, np.float64, order="C")
    e = np.array(ev4, np.float64, order="C")
    a = np.ascontiguousarray(np.asarray(acc3, np.float64)[:, :3])
    _load().oracle_integrate(_p(p), _p(v), _p(e), _p(a), len(p), _ref(params))
    return p, v, e


def step(pos4, vel4, ev4, params, n_steps: int = 1):
    """Full FP64 frames; returns the sorted FP64 state (pos4, vel4, ev4)."""
    p = np.array(pos4, np.float64, order="C")
    v = np.array(vel4, np.float64, order="C")
    e = np.array(ev4, np.float64, order="C")
    lib = _load()
    for _ in range(n_steps):
        r = lib.oracle_step(_p(p), _p(v), _p(e), len(p), _ref(params))
        if r < 0:
            raise MemoryError("oracle_step allocation failed")
    return p, v, e


def max_threads_env() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", "0") or 0)
