"""Record golden fixtures from the reference's own CUDA kernels.

Runs on a GPU machine where oracle/_ref/ holds the reference harness (built by
__graft_entry__.build() from the reference's sources). For each scene below it
runs one reference frame (arrange, density, force, integrate) through the
harness and saves the input state and every intermediate array into
tests/golden/<scene>.npz. tests/test_golden.py checks the CPU oracle against
these fixtures; tests/test_gpu_golden.py checks the GB300 library.

    python tests/golden/make_golden.py --out tests/golden
    python tests/golden/make_golden.py --bench [--frames 200]

--bench instead times the reference's benchmark loop (its runBenchmark) on
the 3.94M-particle scenes and prints one JSON line per scene.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import __graft_entry__ as ge  # noqa: E402
from gpu_helpers import dam_scene, dense_scene, shuffled  # noqa: E402


def mixed_scene(g, seed=7):
    """A dense block (reference default spacing) inside a sparse jittered
    lattice: TRA and SMS cells side by side, with every branch of the
    performance model."""
    text = '''{"fluid_block": [], "mass": 0.00027, "interval": 0.15,
               "xx": 0.5, "yy": 0.5, "zz": 0.5}'''
    s = g.parse_scene(text)
    p = g.params_init(s)
    rng = np.random.default_rng(seed)
    step_d = 0.0045
    a = 0.16 + np.arange(14) * step_d
    dense = np.stack(np.meshgrid(a, a, a, indexing="ij"), -1).reshape(-1, 3)
    dense += rng.uniform(-0.1, 0.1, dense.shape) * step_d
    b = 0.07 + np.arange(16) * 0.021
    sparse = np.stack(np.meshgrid(b, b, b, indexing="ij"), -1).reshape(-1, 3)
    sparse += rng.uniform(-0.2, 0.2, sparse.shape) * 0.021
    lo, hi = a[0] - 0.01, a[-1] + 0.01
    keep = ~np.all((sparse > lo) & (sparse < hi), axis=1)
    pts = np.concatenate([dense, sparse[keep]]).astype(np.float32)
    pos = np.zeros((len(pts), 4), np.float32)
    pos[:, :3] = pts
    return s, p, pos


def scenes(g):
    out = {}
    s, p, pos = dam_scene(g, n_side=16)
    out["sparse_dam"] = (p, shuffled(pos, seed=21))
    s, p, pos = dense_scene(g, n_side=18)
    out["dense_default"] = (p, shuffled(pos, seed=22))
    s, p, pos = mixed_scene(g)
    out["mixed"] = (p, shuffled(pos, seed=23))
    # 32^3 = 32,768 particles of the 262,144-particle dam break (64^3, seed 0):
    # the same physics and proportions at half the size (column in the lower
    # left quarter of a 1.28 x 0.64 x 0.64 m box)
    s, p, pos = dam_scene(g, n_side=32, box=(1.28, 0.64, 0.64), seed=0)
    out["dam_32k"] = (p, shuffled(pos, seed=24))
    return out


def params_bytes(p) -> np.ndarray:
    return np.frombuffer(ctypes.string_at(ctypes.addressof(p), ctypes.sizeof(p)), np.uint8)


def record(out_dir: Path, only=None):
    from oracle import refharness as rh
    g = ge.package()
    out_dir.mkdir(parents=True, exist_ok=True)
    rng = np.random.default_rng(5)
    for name, (p, pos) in scenes(g).items():
        vel = np.zeros_like(pos)
        vel[:, :3] = rng.normal(0.0, 0.3, (len(pos), 3))
        if only and name not in only:
            continue   # the velocities are drawn all the same: one stream
        ev = vel.copy()
        r = rh.run_tick(p, pos, vel, ev)
        mi, ms, mc = r["micro_index"], r["micro_start"], r["micro_count"]
        np.savez_compressed(
            out_dir / f"{name}.npz",
            params=params_bytes(p), in_pos=pos, in_vel=vel, in_ev=ev,
            hash=r["hash"], cell_offset=r["cell_offset"], cell_nump=r["cell_nump"],
            micro_index=mi, micro_start=ms, micro_count=mc,
            micro_total=np.int64(r["micro_total"]),
            block_req=r["block_req"], index=r["index"],
            middle=np.int32(r["middle"]), task_count=np.int32(r["task_count"]),
            tasks=r["tasks"], sorted_pos=r["sorted_pos"], sorted_vel=r["sorted_vel"],
            sorted_ev=r["sorted_ev"], density_pos=r["density_pos"],
            density_ev=r["density_ev"], force_acc=r["force_acc"],
            final_pos=r["final_pos"], final_vel=r["final_vel"], final_ev=r["final_ev"])
        print(f"{name}: n={len(pos)} middle={r['middle']} tasks={r['task_count']} "
              f"sms_cells={(r['block_req'] > 0).sum()}")


def bench(frames: int):
    from oracle import refharness as rh
    g = ge.package()
    for scene in ("scene_default.json", "dam_break_3_94m.json", "dam_break_262k.json"):
        s = g.load_scene(g.scene_path(scene))
        p = g.params_init(s)
        pos = g.lattice(s, p)
        r = rh.run_bench(p, pos, frames)
        r["scene"] = scene
        print(json.dumps(r), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(Path(__file__).resolve().parent))
    ap.add_argument("--bench", action="store_true")
    ap.add_argument("--frames", type=int, default=200)
    ap.add_argument("--only", nargs="*", help="record only these scenes")
    a = ap.parse_args()
    ge.build()
    if a.bench:
        bench(a.frames)
    else:
        record(Path(a.out), a.only)


if __name__ == "__main__":
    main()
