"""Python driver of the reference-kernel harness (test infrastructure only).

run_tick() runs one reference frame (arrange, density, force, integrate) on a
given state with the reference's own kernels and returns every intermediate
array; run_frames() steps whole frames and returns the final state;
run_bench() runs the reference's benchmark loop and returns its report.
Both need a GPU and oracle/_ref/ (see build_ref.py).
"""
from __future__ import annotations

import json
import subprocess
import tempfile
from pathlib import Path

import numpy as np

from .build_ref import CUBIN, HARNESS

TASK_DTYPE = np.dtype([
    ("is_same", np.int8), ("pad_", np.uint8), ("paired_bounds", np.uint16),
    ("cellid", np.int32), ("cell_pos", np.uint16, (3,)), ("p_offset", np.uint16),
    ("xxi", np.int8), ("xxx", np.int8), ("yyi", np.int8), ("yyy", np.int8),
    ("zzi", np.int8), ("zzz", np.int8),
    ("cell_begin", np.int32), ("cell_particle_count", np.int32),
], align=True)


def available() -> bool:
    return CUBIN.exists() and HARNESS.exists()


def write_input(path: Path, params, pos4, vel4=None, ev4=None) -> None:
    import ctypes
    pos = np.ascontiguousarray(pos4, np.float32).reshape(-1, 4)
    n = len(pos)
    vel = np.zeros_like(pos) if vel4 is None else np.ascontiguousarray(vel4, np.float32)
    ev = np.zeros_like(pos) if ev4 is None else np.ascontiguousarray(ev4, np.float32)
    with open(path, "wb") as f:
        f.write(b"GSPHREF1")
        f.write(ctypes.string_at(ctypes.addressof(params), ctypes.sizeof(params)))
        f.write(np.int32(n).tobytes())
        f.write(pos.tobytes())
        f.write(vel.reshape(n, 4).tobytes())
        f.write(ev.reshape(n, 4).tobytes())


def _read_dir(d: Path) -> dict:
    out = {}
    for line in (d / "meta.txt").read_text().splitlines():
        f = line.split()
        if len(f) == 2:
            out[f[0]] = int(f[1])
            continue
        name, dtype, rows, cols = f[0], f[1], int(f[2]), int(f[3])
        raw = (d / f"{name}.bin").read_bytes()
        if dtype == "task":
            a = np.frombuffer(raw, TASK_DTYPE).copy()
        else:
            a = np.frombuffer(raw, np.dtype(dtype)).copy()
            if cols > 1:
                a = a.reshape(rows, cols)
        out[name] = a
    return out


def run_tick(params, pos4, vel4=None, ev4=None, timeout=600) -> dict:
    if not available():
        raise RuntimeError("reference harness not built (oracle/_ref)")
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        write_input(td / "in.bin", params, pos4, vel4, ev4)
        (td / "out").mkdir()
        subprocess.run([str(HARNESS), str(CUBIN), "tick", str(td / "in.bin"),
                        str(td / "out")], check=True, timeout=timeout)
        return _read_dir(td / "out")


def run_frames(params, pos4, frames: int, timeout=1800) -> dict:
    """final_pos (n, 4), final_vel (n, 3), final_ev (n, 4) after `frames`
    reference frames from the given positions at rest."""
    if not available():
        raise RuntimeError("reference harness not built (oracle/_ref)")
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        write_input(td / "in.bin", params, pos4)
        (td / "out").mkdir()
        subprocess.run([str(HARNESS), str(CUBIN), "run", str(td / "in.bin"), str(frames),
                        str(td / "out")], check=True, timeout=timeout)
        return _read_dir(td / "out")


def run_bench(params, pos4, frames: int, timeout=1800) -> dict:
    if not available():
        raise RuntimeError("reference harness not built (oracle/_ref)")
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        write_input(td / "in.bin", params, pos4)
        r = subprocess.run([str(HARNESS), str(CUBIN), "bench", str(td / "in.bin"),
                            str(frames)], check=True, timeout=timeout,
                           capture_output=True, text=True)
        return json.loads(r.stdout.strip().splitlines()[-1])
