"""GB300-native weakly-compressible SPH step: Python mirror of the reference's
host interface over the C ABI in include/gsph.h.

`HybridSystem` mirrors sph::HybridSystem of KemengHuang/Fast-General-GPU-SPH-
framework (src/simulation/sph_hybrid_system.h:46-137): it is built from a scene
JSON file (or from arrays), `tick()` advances one frame (arrange, density,
force, integrate) and `runBenchmark(frames)` is the headless benchmark with the
reference's report fields. Every call goes through libgsph.so (hand-written
sm_103a CUDA); there is no CPU fallback — if the library is missing or no GPU
is visible, construction raises GsphError.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "lib" / "libgsph.so"
SCENES_DIR = PKG_DIR / "scenes"
MAX_FLUID_BLOCKS = 64

# gsph_status codes
OK = 0
ERR_INVALID_ARG = -1
ERR_IO = -2
ERR_PARSE = -3
ERR_CUDA = -4
ERR_OUT_OF_MEMORY = -5
ERR_CAPACITY = -6
ERR_DOMAIN = -7
ERR_NO_DEVICE = -8
ERR_STATE = -9

# gsph_field
FIELD_POSITION = 0
FIELD_VELOCITY = 1
FIELD_EVAL_VELOCITY = 2
FIELD_ACCELERATION = 3
FIELD_KEY = 4
FIELD_PERMUTATION = 5
FIELD_CELL_START = 6
FIELD_CELL_COUNT = 7
FIELD_MICRO_START = 8
FIELD_BLOCK_REQ = 9
FIELD_COMPACT_INDEX = 10
FIELD_TASKS = 11
FIELD_SPLIT = 12
FIELD_COLOR = 13
FIELD_FINAL_POSITION = 14
FIELD_NEIGHBOR_COUNT = 15

# gsph_viscosity_model
VISCOSITY_LAPLACIAN = 0
VISCOSITY_ARTIFICIAL = 1


class GsphError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"gsph error {status}: {message}")
        self.status = status


class Scene(C.Structure):
    _fields_ = [
        ("world", C.c_float * 3),
        ("mass", C.c_float),
        ("interval", C.c_float),
        ("recomm_nump", C.c_uint32),
        ("n_blocks", C.c_uint32),
        ("block_begin", (C.c_float * 3) * MAX_FLUID_BLOCKS),
        ("block_end", (C.c_float * 3) * MAX_FLUID_BLOCKS),
        ("kernel", C.c_float),
        ("rest_density", C.c_float),
        ("gas_constant", C.c_float),
        ("viscosity", C.c_float),
        ("time_step", C.c_float),
        ("gravity_y", C.c_float),
        ("jitter", C.c_float),
        ("seed", C.c_uint64),
    ]


class Params(C.Structure):
    _fields_ = [
        ("world_size", C.c_float * 3),
        ("cell_size", C.c_float), ("inv_cell_size", C.c_float),
        ("grid_size", C.c_int32 * 3),
        ("kernel", C.c_float), ("kernel_2", C.c_float), ("mass", C.c_float),
        ("gravity", C.c_float * 3),
        ("wall_damping", C.c_float), ("rest_density", C.c_float),
        ("gas_constant", C.c_float), ("viscosity", C.c_float),
        ("time_step", C.c_float),
        ("surface_normal", C.c_float), ("surface_coe", C.c_float),
        ("poly6_value", C.c_float), ("spiky_value", C.c_float),
        ("visco_value", C.c_float), ("grad_poly6", C.c_float),
        ("lplc_poly6", C.c_float),
        ("self_density", C.c_float),
        ("inv_rest_density", C.c_float), ("density_scale", C.c_float),
        ("half_spiky_value", C.c_float),
        ("viscosity_visco_value", C.c_float), ("grad_color_scale", C.c_float),
        ("lplc_color_scale", C.c_float),
        ("bound_interval", C.c_float), ("bound_min", C.c_float * 3),
        ("bound_max", C.c_float * 3),
    ]

    @property
    def numc(self) -> int:
        g = self.grid_size
        return int(g[0]) * int(g[1]) * int(g[2])


class BlockTask(C.Structure):
    _fields_ = [
        ("is_same", C.c_int8), ("pad_", C.c_uint8), ("paired_bounds", C.c_uint16),
        ("cellid", C.c_int32), ("cell_pos", C.c_uint16 * 3),
        ("p_offset", C.c_uint16),
        ("xxi", C.c_int8), ("xxx", C.c_int8), ("yyi", C.c_int8),
        ("yyy", C.c_int8), ("zzi", C.c_int8), ("zzz", C.c_int8),
        ("cell_begin", C.c_int32), ("cell_particle_count", C.c_int32),
    ]


BLOCK_TASK_DTYPE = np.dtype([
    ("is_same", np.int8), ("pad_", np.uint8), ("paired_bounds", np.uint16),
    ("cellid", np.int32), ("cell_pos", np.uint16, (3,)), ("p_offset", np.uint16),
    ("xxi", np.int8), ("xxx", np.int8), ("yyi", np.int8), ("yyy", np.int8),
    ("zzi", np.int8), ("zzz", np.int8),
    ("cell_begin", np.int32), ("cell_particle_count", np.int32),
], align=True)
assert BLOCK_TASK_DTYPE.itemsize == 32 == C.sizeof(BlockTask)


class Info(C.Structure):
    _fields_ = [
        ("n_particles", C.c_uint32), ("n_cells", C.c_uint32),
        ("grid_size", C.c_int32 * 3),
        ("tra_particles", C.c_int32), ("sms_tasks", C.c_int32),
        ("occupied_cells", C.c_int32), ("big_cells", C.c_int32),
        ("frames", C.c_uint64), ("device_bytes", C.c_uint64),
        ("n_scenes", C.c_uint32), ("reserved_", C.c_uint32),
    ]


class Tuning(C.Structure):
    """gsph_tuning: split thresholds, CTAs per SM of the density/force kernels
    and their warps per block (defaults: the reference's 96 / 15 / 60,
    6 / 4 / 4 / 4 CTAs of 8 warps)."""
    _fields_ = [(n, C.c_int32) for n in (
        "sparse_total", "sparse_self", "mid_total", "ctas_density_tra",
        "ctas_density_sms", "ctas_force_tra", "ctas_force_sms", "warps_per_block")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class ServerConfig(C.Structure):
    """gsph_server_config."""
    _fields_ = [("budget_bytes", C.c_uint64), ("particle_capacity", C.c_uint64),
                ("cell_capacity", C.c_uint64), ("scene_capacity", C.c_uint32),
                ("chunk_frames", C.c_int32), ("device", C.c_int32), ("max_batches", C.c_int32)]


class ServerStats(C.Structure):
    """gsph_server_stats."""
    _fields_ = [(n, C.c_uint64) for n in (
        "submitted", "finished", "rejected", "frames", "chunks", "particle_steps",
        "queued", "resident", "resident_particles", "resident_bytes", "batches")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class BenchReport(C.Structure):
    _fields_ = [
        ("measured_frames", C.c_int32), ("warmup_frames", C.c_int32),
        ("total_wall_ms", C.c_double), ("avg_frame_ms", C.c_double),
        ("fps", C.c_double), ("checksum", C.c_double * 5),
        ("tra_particles", C.c_int32), ("sms_tasks", C.c_int32),
        ("is_same_pairs", C.c_int32), ("total_pairs", C.c_int32),
        ("same_cell_pairs", C.c_int32), ("full_is_same_pairs", C.c_int32),
        ("partial_is_same_pairs", C.c_int32), ("compact_is_same_pairs", C.c_int32),
        ("widened_is_same_pairs", C.c_int32),
        ("arrange_ms", C.c_double), ("density_ms", C.c_double),
        ("force_ms", C.c_double), ("integrate_ms", C.c_double),
        ("total_kernel_ms", C.c_double), ("particle_steps_per_s", C.c_double),
    ]


# Exported symbols with their ctypes signatures (argtypes, restype).
_VP = C.c_void_p
_SIGS = {
    "gsph_last_error": ([], C.c_char_p),
    "gsph_abi_version": ([], C.c_int),
    "gsph_scene_default": ([C.POINTER(Scene)], C.c_int),
    "gsph_scene_load_json": ([C.c_char_p, C.POINTER(Scene)], C.c_int),
    "gsph_scene_parse_json": ([C.c_char_p, C.c_size_t, C.POINTER(Scene)], C.c_int),
    "gsph_params_init": ([C.POINTER(Scene), C.POINTER(Params)], C.c_int),
    "gsph_lattice_count": ([C.POINTER(Scene), C.POINTER(Params), C.POINTER(C.c_uint32)], C.c_int),
    "gsph_lattice_fill": ([C.POINTER(Scene), C.POINTER(Params), _VP, C.c_uint32,
                           C.POINTER(C.c_uint32)], C.c_int),
    "gsph_create": ([C.POINTER(Params), _VP, _VP, C.c_uint32, C.c_int, C.POINTER(_VP)], C.c_int),
    "gsph_create_from_json": ([C.c_char_p, C.c_int, C.POINTER(_VP)], C.c_int),
    "gsph_destroy": ([_VP], C.c_int),
    "gsph_snapshot_save": ([_VP, C.c_char_p], C.c_int),
    "gsph_snapshot_load": ([C.c_char_p, C.c_int, C.POINTER(_VP)], C.c_int),
    "gsph_snapshot_info": ([C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64),
                            C.POINTER(C.c_uint64)], C.c_int),
    "gsph_batch_create": ([C.POINTER(Params), C.POINTER(C.c_uint32), C.c_uint32, _VP, _VP,
                           C.c_int, C.POINTER(_VP)], C.c_int),
    "gsph_batch_ranges": ([_VP, _VP, _VP], C.c_int),
    "gsph_batch_create_ex": ([C.POINTER(Params), C.POINTER(C.c_uint32), C.c_uint32, _VP, _VP,
                              C.c_uint64, C.c_uint64, C.c_uint32, C.c_int, C.POINTER(_VP)],
                             C.c_int),
    "gsph_batch_repack": ([_VP, _VP, C.c_uint32, _VP, _VP, C.c_uint32, _VP, _VP], C.c_int),
    "gsph_copy_out_scene": ([_VP, C.c_uint32, C.c_int, _VP, C.c_size_t], C.c_int),
    "gsph_step": ([_VP, C.c_int], C.c_int),
    "gsph_arrange": ([_VP], C.c_int),
    "gsph_density": ([_VP], C.c_int),
    "gsph_force": ([_VP], C.c_int),
    "gsph_advance": ([_VP], C.c_int),
    "gsph_step_host_async": ([_VP, C.c_int, _VP, _VP, _VP], C.c_int),
    "gsph_set_graph_mode": ([_VP, C.c_int], C.c_int),
    "gsph_sync": ([_VP], C.c_int),
    "gsph_stream": ([_VP, C.POINTER(_VP)], C.c_int),
    "gsph_get_info": ([_VP, C.POINTER(Info)], C.c_int),
    "gsph_get_params": ([_VP, C.POINTER(Params)], C.c_int),
    "gsph_copy_out": ([_VP, C.c_int, _VP, C.c_size_t], C.c_int),
    "gsph_copy_in": ([_VP, C.c_int, _VP, C.c_size_t], C.c_int),
    "gsph_copy_in_async": ([_VP, C.c_int, _VP, C.c_size_t], C.c_int),
    "gsph_copy_out_async": ([_VP, C.c_int, _VP, C.c_size_t], C.c_int),
    "gsph_checksum": ([_VP, C.POINTER(C.c_double)], C.c_int),
    "gsph_tuning_default": ([C.POINTER(Tuning)], C.c_int),
    "gsph_server_create": ([C.POINTER(ServerConfig), C.POINTER(_VP)], C.c_int),
    "gsph_server_destroy": ([_VP], C.c_int),
    "gsph_server_submit": ([_VP, C.c_uint64, C.POINTER(Params), _VP, _VP, C.c_uint32,
                            C.c_uint32], C.c_int),
    "gsph_server_step": ([_VP, C.POINTER(C.c_int)], C.c_int),
    "gsph_server_poll": ([_VP, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)], C.c_int),
    "gsph_server_take": ([_VP, C.c_uint64, _VP, _VP], C.c_int),
    "gsph_server_get_stats": ([_VP, C.POINTER(ServerStats)], C.c_int),
    "gsph_set_render_transform": ([_VP, C.POINTER(C.c_float), C.POINTER(C.c_float)], C.c_int),
    "gsph_get_tuning": ([_VP, C.POINTER(Tuning)], C.c_int),
    "gsph_set_tuning": ([_VP, C.POINTER(Tuning)], C.c_int),
    "gsph_set_viscosity_model": ([_VP, C.c_int, C.c_float, C.c_float], C.c_int),
    "gsph_autotune": ([_VP, C.c_int, C.POINTER(Tuning), C.c_int, C.POINTER(Tuning),
                       C.POINTER(C.c_float)], C.c_int),
    "gsph_reductions": ([_VP, C.POINTER(C.c_double)], C.c_int),
    "gsph_benchmark": ([_VP, C.c_int, C.POINTER(BenchReport)], C.c_int),
    "gsph_set_stage_timing": ([_VP, C.c_int], C.c_int),
    "gsph_stage_times": ([_VP, C.POINTER(C.c_float)], C.c_int),
    "gsph_grid_sort_scratch_bytes": ([C.c_uint32, C.c_uint32], C.c_size_t),
    "gsph_grid_sort_dev": ([C.POINTER(Params), C.c_uint32, _VP, _VP, _VP, _VP, _VP, _VP,
                            _VP, _VP, _VP, _VP, C.c_size_t, _VP], C.c_int),
    "gsph_grid_sort_dev_noalloc": ([C.POINTER(Params), C.c_uint32, _VP, _VP, _VP, _VP, _VP,
                                    _VP, _VP, _VP, _VP, _VP], C.c_int),
}

_lib = None


def load_library(path: os.PathLike | str | None = None) -> C.CDLL:
    """Load libgsph.so (built by build.py); raise GsphError if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise GsphError(ERR_STATE, f"CUDA library not built: {p} (run __graft_entry__.build())")
    lib = C.CDLL(str(p))
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if path is None:
        _lib = lib
    return lib


def _check(status: int) -> None:
    if status != OK:
        msg = load_library().gsph_last_error()
        raise GsphError(status, msg.decode() if msg else "")


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# ---------------------------------------------------------------- scenes ----
def scene_default() -> Scene:
    s = Scene()
    _check(load_library().gsph_scene_default(C.byref(s)))
    return s


def load_scene(path: os.PathLike | str) -> Scene:
    """readSceneFromJsonFile (sph_hybrid_system.cpp:69-126)."""
    s = Scene()
    _check(load_library().gsph_scene_load_json(str(path).encode(), C.byref(s)))
    return s


def parse_scene(text: str | bytes) -> Scene:
    b = text.encode() if isinstance(text, str) else text
    s = Scene()
    _check(load_library().gsph_scene_parse_json(b, len(b), C.byref(s)))
    return s


def params_init(scene: Scene) -> Params:
    """defaultInitializeSPHSysPara (sph_hybrid_system.cpp:127-202)."""
    p = Params()
    _check(load_library().gsph_params_init(C.byref(scene), C.byref(p)))
    return p


def lattice(scene: Scene, params: Params) -> np.ndarray:
    """Initial particle lattice (initializeScene, sph_hybrid_system.cpp:441-464)
    as an (N, 4) float32 array, w = 0."""
    lib = load_library()
    n = C.c_uint32()
    _check(lib.gsph_lattice_count(C.byref(scene), C.byref(params), C.byref(n)))
    out = np.zeros((max(n.value, 1), 4), np.float32)
    got = C.c_uint32()
    _check(lib.gsph_lattice_fill(C.byref(scene), C.byref(params), _ptr(out), n.value,
                                 C.byref(got)))
    return out[: got.value].copy()


def scene_path(name: str) -> Path:
    return SCENES_DIR / name


# ---------------------------------------------------------------- system ----
class HybridSystem:
    """One scene on one GPU (mirror of sph::HybridSystem)."""

    def __init__(self, scene: os.PathLike | str | None = None, *,
                 params: Params | None = None, positions: np.ndarray | None = None,
                 velocities: np.ndarray | None = None, device: int = 0):
        lib = load_library()
        h = C.c_void_p()
        if scene is not None:
            _check(lib.gsph_create_from_json(str(scene).encode(), device, C.byref(h)))
        else:
            if params is None or positions is None:
                raise ValueError("give a scene path or params + positions")
            pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
            vel = None
            if velocities is not None:
                vel = np.ascontiguousarray(velocities, np.float32).reshape(-1, 4)
                if vel.shape != pos.shape:
                    raise ValueError("velocities must match positions")
            _check(lib.gsph_create(C.byref(params), _ptr(pos),
                                   _ptr(vel) if vel is not None else None,
                                   pos.shape[0], device, C.byref(h)))
        self._h = h
        self._lib = lib
        self.params = Params()
        _check(lib.gsph_get_params(h, C.byref(self.params)))
        self.n = int(self.info().n_particles)

    # lifetime
    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.gsph_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # frame
    def tick(self) -> None:
        _check(self._lib.gsph_step(self._h, 1))

    def step(self, n: int = 1) -> None:
        _check(self._lib.gsph_step(self._h, n))

    def arrange(self) -> None:
        _check(self._lib.gsph_arrange(self._h))

    def density(self) -> None:
        _check(self._lib.gsph_density(self._h))

    def force(self) -> None:
        _check(self._lib.gsph_force(self._h))

    def advance(self) -> None:
        _check(self._lib.gsph_advance(self._h))

    def sync(self) -> None:
        _check(self._lib.gsph_sync(self._h))

    def stream(self) -> int:
        """The handle's cudaStream_t as an integer."""
        out = C.c_void_p()
        _check(self._lib.gsph_stream(self._h, C.byref(out)))
        return int(out.value or 0)

    def copy_in_async(self, field: int, host_ptr: int, nbytes: int) -> None:
        _check(self._lib.gsph_copy_in_async(self._h, field, host_ptr, nbytes))

    def step_host_async(self, frames: int, pos_ptr: int, vel_ptr: int, ev_ptr: int) -> None:
        """gsph_step_host_async: pinned host state in, `frames` frames, state out
        into the same arrays (complete after sync())."""
        _check(self._lib.gsph_step_host_async(self._h, int(frames), pos_ptr, vel_ptr, ev_ptr))

    def copy_out_async(self, field: int, host_ptr: int, nbytes: int) -> None:
        _check(self._lib.gsph_copy_out_async(self._h, field, host_ptr, nbytes))

    def set_graph_mode(self, frames) -> None:
        """frames > 0: step through CUDA graphs of that many frames; 0 or
        False: launch kernel by kernel (True means one frame per graph)."""
        _check(self._lib.gsph_set_graph_mode(self._h, int(frames)))

    def set_stage_timing(self, on: bool) -> None:
        _check(self._lib.gsph_set_stage_timing(self._h, int(bool(on))))

    def stage_times(self) -> dict:
        out = (C.c_float * 4)()
        _check(self._lib.gsph_stage_times(self._h, out))
        return dict(zip(("arrange", "density", "force", "integrate"), map(float, out)))

    # reference getters
    def getNumParticles(self) -> int:
        return self.n

    def getPosition(self, i: int) -> np.ndarray:
        return self.copy_out(FIELD_POSITION)[i, :3].copy()

    def info(self) -> Info:
        out = Info()
        _check(self._lib.gsph_get_info(self._h, C.byref(out)))
        return out

    # data movement
    def copy_out(self, field: int) -> np.ndarray:
        numc = self.params.numc
        n = self.n
        if field in (FIELD_POSITION, FIELD_VELOCITY, FIELD_EVAL_VELOCITY, FIELD_ACCELERATION,
                     FIELD_FINAL_POSITION):
            out = np.empty((n, 4), np.float32)
        elif field in (FIELD_KEY, FIELD_COLOR):
            out = np.empty(n, np.uint32)
        elif field in (FIELD_PERMUTATION, FIELD_COMPACT_INDEX, FIELD_NEIGHBOR_COUNT):
            out = np.empty(n, np.int32)
        elif field == FIELD_CELL_START:
            out = np.empty(numc + 1, np.int32)
        elif field in (FIELD_CELL_COUNT, FIELD_BLOCK_REQ):
            out = np.empty(numc, np.int32)
        elif field == FIELD_MICRO_START:
            out = np.empty(numc * 64 + 1, np.int32)
        elif field == FIELD_SPLIT:
            out = np.empty(2, np.int32)
        elif field == FIELD_TASKS:
            split = self.copy_out(FIELD_SPLIT)
            t = int(split[1])
            out = np.empty(t + (t & 1), BLOCK_TASK_DTYPE)
        else:
            raise ValueError(f"unknown field {field}")
        _check(self._lib.gsph_copy_out(self._h, field, _ptr(out) if out.size else
                                       _ptr(np.empty(1, np.uint8)), out.nbytes))
        return out

    def copy_in(self, field: int, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr, np.float32).reshape(-1, 4)
        _check(self._lib.gsph_copy_in(self._h, field, _ptr(a), a.nbytes))

    def checksum(self) -> tuple:
        out = (C.c_double * 5)()
        _check(self._lib.gsph_checksum(self._h, out))
        return tuple(out)

    def reductions(self) -> dict:
        out = (C.c_double * 8)()
        _check(self._lib.gsph_reductions(self._h, out))
        keys = ("mass", "px", "py", "pz", "kinetic", "sx", "sy", "sz")
        return dict(zip(keys, out))

    def set_render_transform(self, ratio=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0)) -> None:
        """gsph_set_render_transform: FIELD_FINAL_POSITION = pos * ratio + origin."""
        r = (C.c_float * 3)(*ratio)
        o = (C.c_float * 3)(*origin)
        _check(self._lib.gsph_set_render_transform(self._h, r, o))

    def set_viscosity_model(self, model: int, alpha: float = 0.0, c0: float = 0.0) -> None:
        """VISCOSITY_LAPLACIAN (the reference's, the default) or
        VISCOSITY_ARTIFICIAL (Monaghan's artificial viscosity with alpha and
        the speed of sound c0) for every scene of this handle."""
        _check(self._lib.gsph_set_viscosity_model(self._h, int(model), float(alpha),
                                                  float(c0)))

    def get_tuning(self) -> Tuning:
        t = Tuning()
        _check(self._lib.gsph_get_tuning(self._h, C.byref(t)))
        return t

    def set_tuning(self, t: Tuning) -> None:
        _check(self._lib.gsph_set_tuning(self._h, C.byref(t)))

    def autotune(self, frames_per_trial: int = 3, candidates=None):
        """gsph_autotune: times the candidates (None: the built-in grid) on the
        current state, installs the fastest; returns (Tuning, ms per frame)."""
        best, ms = Tuning(), C.c_float()
        if candidates is None:
            arr, n = None, 0
        else:
            arr = (Tuning * len(candidates))(*candidates)
            n = len(candidates)
        _check(self._lib.gsph_autotune(self._h, frames_per_trial, arr, n, C.byref(best),
                                       C.byref(ms)))
        return best, ms.value

    def save_snapshot(self, path: os.PathLike | str) -> None:
        """gsph_snapshot_save: the state, parameters and frame counter."""
        _check(self._lib.gsph_snapshot_save(self._h, str(path).encode()))

    def runBenchmark(self, frames: int) -> dict:
        r = BenchReport()
        _check(self._lib.gsph_benchmark(self._h, frames, C.byref(r)))
        d = {k: getattr(r, k) for k, _ in BenchReport._fields_}
        d["checksum"] = tuple(r.checksum)
        return d

    @property
    def handle(self) -> int:
        return self._h.value


def tuning_default() -> Tuning:
    t = Tuning()
    _check(load_library().gsph_tuning_default(C.byref(t)))
    return t


def occupancy_signature(cell_count: np.ndarray, n_particles: int) -> tuple:
    """Occupancy histogram of the occupied cells in power-of-two bins (1,
    2-3, 4-7, ..., >= 512), as fractions rounded to 0.05, with the particle
    count's power of two: the key under which Autotuner caches a tuning."""
    occ = np.asarray(cell_count)[np.asarray(cell_count) > 0]
    if occ.size == 0:
        return (0,)
    b = np.minimum(np.floor(np.log2(occ)).astype(np.int64), 9)
    h = np.bincount(b, minlength=10) / occ.size
    return (int(np.log2(max(n_particles, 1))),) + tuple(float(round(x * 20) / 20) for x in h)


class Autotuner:
    """Tunings per occupancy histogram: the first handle with a new signature
    is autotuned (gsph_autotune), later ones with the same signature get the
    cached result without any trial frames."""

    def __init__(self, frames_per_trial: int = 3, candidates=None):
        self.frames = frames_per_trial
        self.candidates = candidates
        self.cache: dict[tuple, tuple[Tuning, float]] = {}

    def signature(self, h: "HybridSystem") -> tuple:
        h.arrange()
        return occupancy_signature(h.copy_out(FIELD_CELL_COUNT), h.n)

    def tune(self, h: "HybridSystem") -> tuple[Tuning, float, bool]:
        """Returns (tuning, ms per frame at tuning time, came from the cache)."""
        sig = self.signature(h)
        if sig in self.cache:
            t, ms = self.cache[sig]
            h.set_tuning(t)
            return t, ms, True
        t, ms = h.autotune(self.frames, self.candidates)
        self.cache[sig] = (t, ms)
        return t, ms, False


class NativeSceneServer:
    """The native continuous-batching server (gsph_server_*): submit requests
    from any thread, call step() from one thread, collect finished results
    with results()."""

    def __init__(self, budget_bytes: int, capacity, chunk: int = 10, device: int = 0,
                 max_batches: int = 1):
        """capacity = (particles, cells, scenes) of each batch; up to
        max_batches batches are opened as admissions need them."""
        lib = load_library()
        cfg = ServerConfig(int(budget_bytes), int(capacity[0]), int(capacity[1]),
                           int(capacity[2]), int(chunk), int(device), int(max_batches))
        h = C.c_void_p()
        _check(lib.gsph_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._lib = lib

    def submit(self, rid: int, params: Params, positions, frames: int, velocities=None):
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
        vel = None if velocities is None else np.ascontiguousarray(velocities,
                                                                    np.float32).reshape(-1, 4)
        _check(self._lib.gsph_server_submit(self._h, rid, C.byref(params),
                                            _ptr(pos) if len(pos) else None,
                                            _ptr(vel) if vel is not None and len(vel) else None,
                                            len(pos), int(frames)))

    def step(self) -> int:
        k = C.c_int()
        _check(self._lib.gsph_server_step(self._h, C.byref(k)))
        return k.value

    def results(self) -> dict:
        """All finished requests not yet taken: {id: (positions, velocities)}."""
        out = {}
        rid, n = C.c_uint64(), C.c_uint32()
        while self._lib.gsph_server_poll(self._h, C.byref(rid), C.byref(n)) == OK:
            pos = np.empty((n.value, 4), np.float32)
            vel = np.empty((n.value, 4), np.float32)
            _check(self._lib.gsph_server_take(self._h, rid.value,
                                              _ptr(pos) if n.value else None,
                                              _ptr(vel) if n.value else None))
            out[rid.value] = (pos, vel)
        return out

    def stats(self) -> dict:
        st = ServerStats()
        _check(self._lib.gsph_server_get_stats(self._h, C.byref(st)))
        return st.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.gsph_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def snapshot_info(path: os.PathLike | str) -> dict:
    """Header of a snapshot file: scenes, particles, frames."""
    s, n, f = C.c_uint32(), C.c_uint64(), C.c_uint64()
    _check(load_library().gsph_snapshot_info(str(path).encode(), C.byref(s), C.byref(n),
                                             C.byref(f)))
    return {"n_scenes": s.value, "n_particles": n.value, "frames": f.value}


def load_snapshot(path: os.PathLike | str, device: int = 0):
    """gsph_snapshot_load: a HybridSystem (one scene) or a Batch that
    continues the saved run bit for bit."""
    lib = load_library()
    h = C.c_void_p()
    _check(lib.gsph_snapshot_load(str(path).encode(), device, C.byref(h)))
    info = Info()
    st = lib.gsph_get_info(h, C.byref(info))
    if st:
        lib.gsph_destroy(h)
        _check(st)
    cls = Batch if info.n_scenes > 1 else HybridSystem
    obj = cls.__new__(cls)
    obj._h = h
    obj._lib = lib
    obj.params = Params()
    _check(lib.gsph_get_params(h, C.byref(obj.params)))
    if cls is Batch:
        obj._refresh()
    else:
        obj.n = int(info.n_particles)
    return obj


class Batch(HybridSystem):
    """Several independent scenes stepped together (gsph_batch_create): one
    launch per stage for all of them. Scene k evolves exactly as it would
    alone (bit-identical). `scenes` is a list of (params, positions[,
    velocities]) with a common physical parameter set."""

    def __init__(self, scenes, device: int = 0, capacity=None):
        """capacity: optional (particles, cells, scenes) to reserve for
        repack(); by default the buffers fit the initial scenes exactly."""
        lib = load_library()
        plist, counts, pos_all, vel_all = self._pack(scenes)
        h = C.c_void_p()
        if capacity is None:
            _check(lib.gsph_batch_create(plist, counts, len(scenes),
                                         _ptr(pos_all) if len(pos_all) else None,
                                         _ptr(vel_all) if len(vel_all) else None,
                                         device, C.byref(h)))
        else:
            pc, cc, sc = capacity
            _check(lib.gsph_batch_create_ex(plist, counts, len(scenes),
                                            _ptr(pos_all) if len(pos_all) else None,
                                            _ptr(vel_all) if len(vel_all) else None,
                                            int(pc), int(cc), int(sc), device, C.byref(h)))
        self._h = h
        self._lib = lib
        self.params = Params()
        _check(lib.gsph_get_params(h, C.byref(self.params)))
        self._refresh()

    @staticmethod
    def _pack(scenes):
        S = len(scenes)
        plist = (Params * max(S, 1))()
        counts = (C.c_uint32 * max(S, 1))()
        pos_parts, vel_parts = [], []
        for k, sc in enumerate(scenes):
            p, pos = sc[0], np.ascontiguousarray(sc[1], np.float32).reshape(-1, 4)
            vel = (np.ascontiguousarray(sc[2], np.float32).reshape(-1, 4)
                   if len(sc) > 2 and sc[2] is not None else np.zeros_like(pos))
            C.memmove(C.addressof(plist[k]), C.addressof(p), C.sizeof(Params))
            counts[k] = len(pos)
            pos_parts.append(pos)
            vel_parts.append(vel)
        pos_all = np.concatenate(pos_parts) if pos_parts else np.zeros((0, 4), np.float32)
        vel_all = np.concatenate(vel_parts) if vel_parts else np.zeros((0, 4), np.float32)
        return plist, counts, np.ascontiguousarray(pos_all), np.ascontiguousarray(vel_all)

    def _refresh(self):
        info = self.info()
        self.n = int(info.n_particles)
        self.num_scenes = S = int(info.n_scenes)
        self.pbase = np.empty(S + 1, np.int32)
        self.cbase = np.empty(S + 1, np.int32)
        _check(self._lib.gsph_batch_ranges(self._h, _ptr(self.pbase), _ptr(self.cbase)))

    def repack(self, keep, add_scenes=()) -> None:
        """Keep the listed scenes (in that order), then append add_scenes."""
        keep_a = np.ascontiguousarray(keep, np.uint32)
        plist, counts, pos_all, vel_all = self._pack(list(add_scenes))
        _check(self._lib.gsph_batch_repack(
            self._h, _ptr(keep_a) if len(keep_a) else None, len(keep_a),
            plist, counts, len(add_scenes),
            _ptr(pos_all) if len(pos_all) else None,
            _ptr(vel_all) if len(vel_all) else None))
        self._refresh()

    def copy_out_scene(self, scene: int, field: int) -> np.ndarray:
        n = int(self.pbase[scene + 1] - self.pbase[scene])
        nc = int(self.cbase[scene + 1] - self.cbase[scene])
        if field in (FIELD_POSITION, FIELD_VELOCITY, FIELD_EVAL_VELOCITY, FIELD_ACCELERATION):
            out = np.empty((n, 4), np.float32)
        elif field == FIELD_KEY:
            out = np.empty(n, np.uint32)
        elif field == FIELD_PERMUTATION:
            out = np.empty(n, np.int32)
        elif field == FIELD_CELL_START:
            out = np.empty(nc + 1, np.int32)
        elif field == FIELD_CELL_COUNT:
            out = np.empty(nc, np.int32)
        else:
            raise ValueError(f"field {field} has no per-scene form")
        _check(self._lib.gsph_copy_out_scene(self._h, scene, field,
                                             _ptr(out) if out.size else _ptr(np.empty(1, np.uint8)),
                                             out.nbytes))
        return out
