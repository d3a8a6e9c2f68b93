#!/usr/bin/env python3
"""Benchmark of the WCSPH step on the 3.94M-particle dam break.

One step = one frame of the hot path (grid sort, SMS/TRA split, density,
force, integrate) over all 3,944,312 particles. Prints ONE JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

The GPU arm times K frames, launched as CUDA graphs of 10 frames, with CUDA
events on the scene's own stream (state resident in HBM, 440 MB > L2, so no
L2 flush is needed), takes per-stage times from the frames that follow (stage
events, frame by frame), samples SM clocks
during the timed region, measures the end-to-end rate through the public API
with pinned host buffers, reports the roofline of the dominant kernel and
times the CPU oracle on the host cores as a reported baseline. The same line
carries the metric's batched and served forms as sub-records: 256 uneven
scenes stepped as one batch (100 frames in one CUDA graph, autotuned) against
per-scene loops of the plain path (kernel by kernel and as CUDA graphs of the
same length), and 10 s of Poisson request arrivals through the native
continuous-batching server against the same trace through an executed
per-scene FIFO loop, with p50/p99 completion latency. The reference arm
(--impl reference) times the CPU restatement of the reference's step (the
reference has no CPU path of its own): full FP64 frames of the same scene.
With N > 1 (torchrun), every rank runs an independent replica: the path does
not shard.
"""
from __future__ import annotations

import argparse
import collections
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("particle-steps/s @3.94M (HBM %); batched/served vs per-scene loop; "
          "p99 ms")
SCENE = "dam_break_3_94m.json"
WORKLOAD = ("dam_break_3_94m: 158^3 = 3,944,312 FP32 particles, dx 0.01 m, h 0.02 m, "
            "jitter +-0.05dx, box 4.74x3.16x1.68 m (237x159x84 cells), Tait B=57142.857, "
            "viscosity 0.8, dt 1e-4 s")
LAUNCHES_PER_FRAME = 14   # 5 grid sort + 4 split + 2 density + 2 force + SMS hash


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Ranks:
    """The replica group: one process per GPU under torchrun, joined over
    torch.distributed (NCCL with GPUs, gloo without) for the barrier and the
    max / sum over ranks; a no-op for a single process. Replicas exchange
    nothing else: the path does not shard."""

    def __init__(self, ws: int):
        self.ws = ws
        self.td = None
        if ws > 1:
            import torch
            import torch.distributed as td
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if not td.is_initialized():
                td.init_process_group(backend)
            self.td = td
            self.device = "cuda" if backend == "nccl" else "cpu"

    def barrier(self):
        if self.td:
            self.td.barrier()

    def _reduce(self, x: float, op) -> float:
        if not self.td:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.td.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x: float) -> float:
        return self._reduce(x, self.td.ReduceOp.MAX if self.td else None)

    def sum(self, x: float) -> float:
        return self._reduce(x, self.td.ReduceOp.SUM if self.td else None)

    def close(self):
        if self.td and self.td.is_initialized():
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except (ValueError, KeyError):
            pass
    return 6800.0, "fallback"


def ncu_traffic(kernel: str, workload: str, key: str = ""):
    """Per-launch DRAM bytes of `kernel` (or its `.key` figure) from the
    committed ncu summary of the same workload (`kernel@workload = value`);
    None where no capture of this workload exists."""
    f = ROOT / "profiles" / "traffic_per_launch.txt"
    if not f.exists():
        return None
    name = re.escape(f"{kernel}@{workload}" + (f".{key}" if key else ""))
    for line in f.read_text().splitlines():
        m = re.match(rf"\s*{name}\s*=\s*([0-9.eE+]+)", line)
        if m:
            return float(m.group(1))
    return None


def tile_bytes(cell_count: np.ndarray, grid, n: int):
    """Cell-tile algorithmic bytes of one density and one force launch: every
    occupied cell stages its 27-cell neighbourhood once (16 B per particle for
    density, 32 B for force) and reads/writes its own particles once (24 B and
    44 B per particle)."""
    gx, gy, gz = grid
    c = cell_count.reshape(gz, gy, gx).astype(np.int64)
    pad = np.pad(c, 1)
    n27 = np.zeros_like(c)
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                n27 += pad[dz:dz + gz, dy:dy + gy, dx:dx + gx]
    s = int(n27[c > 0].sum())
    return 16 * s + 24 * n, 32 * s + 44 * n


def load_pkg():
    import __graft_entry__ as ge
    return ge.package()


def cpu_oracle_rate(params, pos, budget_s: float, max_steps: int, vel=None, ev=None):
    """FP64 oracle frames on the given state (all host threads); returns
    (particle-steps/s, steps, particles, threads)."""
    import oracle
    oracle.build()
    P = np.array(pos, np.float64)
    V = np.zeros_like(P) if vel is None else np.array(vel, np.float64)
    E = np.zeros_like(P) if ev is None else np.array(ev, np.float64)
    lib = oracle._load()
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps:
        lib.oracle_step(P.ctypes.data, V.ctypes.data, E.ctypes.data, len(P), oracle._ref(params))
        steps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return len(P) * steps / dt, steps, len(P), oracle.num_threads()


def reference_scene(scene_file: str):
    """Scene, parameters and lattice of a scene file through the oracle alone
    (its JSON reader, parameter and lattice restatements): the CPU reference
    arm loads no part of the GPU library. The package module is imported only
    for its ctypes struct layouts (it loads libgsph.so lazily, not here)."""
    import oracle
    oracle.build()
    g = load_pkg()
    path = ROOT / "fast-general-gpu-sph-framework_gb300" / "scenes" / scene_file
    s = oracle.scene_from_json(path.read_text(), g.Scene)
    p = oracle.params_init(s, g.Params)
    return s, p, oracle.lattice(s, p)


def run_reference(args, ws, rank):
    """The reference's step on the host cores: the FP64 C/OpenMP restatement
    of HybridSystem::tick() (the reference itself has no CPU path), one full
    frame of the whole scene per step on all host threads. When K + W full
    frames would take more than a few minutes, each step is instead a frame of
    the first M particles of the lattice, M sized to fit (stated in the line)."""
    if rank != 0:
        return 0
    import oracle
    s, p, pos_full = reference_scene(args.scene)
    n_full = len(pos_full)
    lib = oracle._load()

    def state(m):
        P = np.array(pos_full[:m], np.float64)
        return P, np.zeros_like(P), np.zeros_like(P)

    # one untimed full frame sizes the run: K + W frames within ~3 minutes
    P, V, E = state(n_full)
    t = time.perf_counter()
    lib.oracle_step(P.ctypes.data, V.ctypes.data, E.ctypes.data, len(P), oracle._ref(p))
    t_full = time.perf_counter() - t
    total = max(1, args.steps + args.warmup)
    budget_s = 180.0
    sample_n = n_full if total * t_full <= budget_s else max(
        65536, int(n_full * budget_s / (total * t_full)))
    if sample_n < n_full:
        P, V, E = state(sample_n)
    for _ in range(args.warmup):
        lib.oracle_step(P.ctypes.data, V.ctypes.data, E.ctypes.data, len(P), oracle._ref(p))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lib.oracle_step(P.ctypes.data, V.ctypes.data, E.ctypes.data, len(P), oracle._ref(p))
    dt = time.perf_counter() - t0
    value = sample_n * args.steps / dt
    if sample_n == n_full:
        sample = (f"every step one FP64 frame of all {n_full} particles, FP64 C/OpenMP "
                  f"restatement of the reference step")
    else:
        sample = (f"every step one FP64 frame of the first {sample_n} of {n_full} particles "
                  f"(K + W full frames would exceed {budget_s:.0f} s), FP64 C/OpenMP "
                  f"restatement of the reference step")
    workload = WORKLOAD if args.scene == SCENE else args.scene
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3 / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded jittered dam-break lattice generated on the host",
        "config": {"workload": workload, "particles": sample_n,
                   "parallelism": "rank 0 only (CPU)"},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s",
                         "cores": oracle.num_threads(), "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def load_workloads():
    import importlib.util
    name = "gsph_gb300.workloads"
    if name in sys.modules:
        return sys.modules[name]
    load_pkg()
    spec = importlib.util.spec_from_file_location(
        name, ROOT / "fast-general-gpu-sph-framework_gb300" / "workloads.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def batched_record(g, W, args, R, rank, local, frames, graph_frames, autotune=True):
    """Batched workload: independent dam-break scenes (N log-uniform in
    [4,096, 262,144], column aspect uniform in [0.5, 2]) stepped as one batch
    with CUDA graphs of `graph_frames` frames (one launch per stage for all
    scenes, autotuned split and launch shapes), against a loop over the same
    scenes with the plain single-scene path, launched kernel by kernel and as
    CUDA graphs of the same length. Returns the measurements as a dict."""
    import torch
    specs = W.batched_scenes(args.scenes, seed=rank)
    scenes = [W.build(g, sp) for sp in specs]
    total = sum(len(pos) for _, pos in scenes)
    b = g.Batch(scenes, device=local)
    b.step(args.warmup)
    b.sync()
    tuned = None
    if autotune:
        t, ms = b.autotune(frames_per_trial=3)
        tuned = {**t.as_dict(), "trial_ms_per_frame": ms}
    b.set_graph_mode(graph_frames)
    b.step(graph_frames)          # captures the graph outside the timed region
    b.sync()
    stream = torch.cuda.ExternalStream(b.stream(), device=torch.device("cuda", local))
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    R.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    t0 = time.perf_counter()
    ev0.record(stream)
    b.step(frames)
    ev1.record(stream)
    ev1.synchronize()
    wall_b = time.perf_counter() - t0
    clk = clocks.stop()
    dev_ms = ev0.elapsed_time(ev1)
    b.set_graph_mode(0)
    b.set_stage_timing(True)
    b.step(10)
    stages = b.stage_times()
    info = b.info()
    b.close()
    dev_ms = R.max(dev_ms)
    total_all = R.sum(total)
    batched = total_all * frames / (dev_ms / 1e3)

    def loop_rate(gf):
        hs = [g.HybridSystem(params=p, positions=pos, device=local) for p, pos in scenes]
        for h in hs:
            h.set_graph_mode(gf)
            h.step(max(args.warmup, gf))   # with graphs: the capture happens here
            h.sync()
        R.barrier()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for h in hs:
            h.step(frames)
            h.sync()
        dt = R.max(time.perf_counter() - t)
        for h in hs:
            h.close()
        return total_all * frames / dt, dt

    loop_plain, t_plain = loop_rate(0)
    loop_graph, t_graph = loop_rate(graph_frames)
    return {
        "value": batched, "unit": "particle-steps/s", "frames": frames,
        "ms_per_frame": dev_ms / frames, "wall_s": wall_b,
        "workload": f"{len(scenes)} scenes per GPU, {total} particles, N log-uniform "
                    f"[4096, 262144], aspect U[0.5, 2], 262k-scene physics, own boxes",
        "scenes": len(scenes), "particles": total, "cells": int(info.n_cells),
        "graph_frames": graph_frames,
        "timing": f"CUDA events around {frames} frames launched as CUDA graphs of "
                  f"{graph_frames} frames; stage times from 10 frames that follow",
        "tuning": tuned if tuned else "reference thresholds, default shapes",
        "split": {"tra_particles": info.tra_particles, "sms_tasks": info.sms_tasks},
        "stages_ms": stages,
        "per_scene_loop": {"value": loop_plain, "unit": "particle-steps/s",
                           "wall_s": t_plain, "launch": "kernel by kernel"},
        "per_scene_loop_graphs": {"value": loop_graph, "unit": "particle-steps/s",
                                  "wall_s": t_graph,
                                  "launch": f"CUDA graphs of {graph_frames} frames"},
        "speedup_vs_loop": batched / loop_plain,
        "speedup_vs_graph_loop": batched / loop_graph,
        "clocks": clk,
        "gpu_launches": LAUNCHES_PER_FRAME * frames,
    }


def run_batched(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    R = Ranks(ws)
    g = load_pkg()
    W = load_workloads()
    rec = batched_record(g, W, args, R, rank, local, args.steps, args.graph_frames,
                         autotune=not args.no_autotune)
    line = {
        "metric": "aggregate particle-steps/s, batched vs per-scene loop",
        "value": rec["value"], "unit": "particle-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": rec["ms_per_frame"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded jittered dam-break columns generated on the host",
        "config": {"workload": "batched: " + rec["workload"],
                   "graph_frames": args.graph_frames, "cells": rec["cells"],
                   "tuning": rec["tuning"]},
        **{k: rec[k] for k in ("stages_ms", "split", "per_scene_loop",
                               "per_scene_loop_graphs", "speedup_vs_loop",
                               "speedup_vs_graph_loop", "clocks", "gpu_launches")},
        "batched_wall_s": rec["wall_s"],
    }
    if rank == 0:
        print(json.dumps(line))
    R.close()
    return 0


def load_serve():
    import importlib.util
    name = "gsph_gb300.serve"
    if name in sys.modules:
        return sys.modules[name]
    load_pkg()
    spec = importlib.util.spec_from_file_location(
        name, ROOT / "fast-general-gpu-sph-framework_gb300" / "serve.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def _builder(g, W, trace, ahead=16):
    """Yields (index, params, positions) of the trace's scenes in order,
    built by a small thread pool up to `ahead` requests in advance (the
    lattice fill releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=4) as pool:
        q = collections.deque()
        nxt = 0
        for i in range(len(trace)):
            while nxt < len(trace) and nxt < i + ahead:
                q.append(pool.submit(W.build, g, trace[nxt][1]))
                nxt += 1
            p, pos = q.popleft().result()
            yield i, p, pos


def fifo_loop_executed(g, W, S, trace, local, graph_frames):
    """The per-scene FIFO loop of the plain single-scene path, executed: the
    requests are served one at a time in arrival order (a request that has not
    arrived yet is waited for), each on its own HybridSystem stepped its K
    frames as CUDA graphs of `graph_frames` frames, with its positions read
    back at the end. Lattices are built ahead by a thread pool (they are the
    request's input, as in the served run)."""
    from types import SimpleNamespace
    done = []
    work = 0
    t0 = time.perf_counter()
    for i, p, pos in _builder(g, W, trace):
        t_arr, sp, k = trace[i]
        wait = t_arr - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        h = g.HybridSystem(params=p, positions=pos, device=local)
        h.set_graph_mode(graph_frames)
        h.step(k)
        h.copy_out(g.FIELD_POSITION)     # result read-back (synchronises)
        h.close()
        done.append(SimpleNamespace(rid=i, t_arrival=t0 + t_arr,
                                    t_done=time.perf_counter()))
        work += len(pos) * k
    makespan = time.perf_counter() - t0
    lat = S.latency_stats(done)
    return {"value": work / makespan, "unit": "particle-steps/s", "latency": lat,
            "makespan_s": makespan, "requests": len(done),
            "method": f"executed: one request at a time in arrival order, each its own "
                      f"HybridSystem stepped K frames as CUDA graphs of {graph_frames} "
                      f"frames, positions read back"}


def served_record(g, W, S, args, R, rank, local, duration):
    """Served workload: Poisson arrivals (50/s) of dam-break requests (N
    log-uniform in [8,192, 1,048,576], K uniform in [50, 500]) replayed in
    real time for `duration` seconds of arrivals. A client thread builds each
    scene when it arrives; the server admits queued requests FIFO between
    chunks of frames while they fit the HBM budget and the batch's capacity,
    steps all resident scenes together and retires each after its K frames
    (its positions are read back). Then the same trace through the executed
    per-scene FIFO loop. Returns the measurements as a dict."""
    trace = W.served_requests(duration, seed=1 + rank)
    budget = int(args.budget_gb * 1e9)
    cap = (args.cap_particles, (1 << 26) - 1, 4096)
    # batches the server may open: as many as the budget holds at their
    # capacity (each batch's key space holds fewer than 2^26 cells)
    batch_bytes = S.scene_bytes(cap[0], cap[1])
    max_batches = args.max_batches or max(1, budget // batch_bytes)
    native = args.server == "native"
    if native:
        srv = g.NativeSceneServer(budget, cap, chunk=args.chunk, device=local,
                                  max_batches=max_batches)
        arrivals, finished = {}, {}
    else:
        srv = S.SceneServer(g, budget_bytes=budget, capacity=cap, chunk=args.chunk,
                            device=local, keep_results=False, max_batches=max_batches)
    # warm the library (context, modules) on a small scene outside the timed run
    p0, pos0 = W.build(g, {"nx": 16, "ny": 16, "nz": 16, "seed": 3})
    with g.HybridSystem(params=p0, positions=pos0, device=local) as h:
        h.step(args.warmup)
        h.sync()

    done_submitting = threading.Event()
    R.barrier()
    t0 = time.perf_counter()
    errors = []

    def client():
        # scenes are built ahead of their arrival and submitted at arrival time
        try:
            for i, p, pos in _builder(g, W, trace):
                t_arr, sp, k = trace[i]
                dt = t0 + t_arr - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                if native:
                    arrivals[i] = (t0 + t_arr, len(pos), k)
                    srv.submit(i, p, pos, k)
                else:
                    srv.submit(S.Request(i, p, pos, k, t0 + t_arr))
        except Exception as e:         # surfaced after the run
            errors.append(e)
        finally:
            done_submitting.set()

    clocks = ClockSampler(local)
    clocks.start()
    th = threading.Thread(target=client, daemon=True)
    th.start()
    busy = 0.0
    peak_resident = 0
    peak_particles = 0
    peak_batches = 0
    if native:
        while True:
            tb = time.perf_counter()
            k = srv.step()
            now = time.perf_counter()
            for rid in srv.results():
                finished[rid] = now
            st = srv.stats()
            peak_resident = max(peak_resident, st["resident"])
            peak_particles = max(peak_particles, st["resident_particles"])
            peak_batches = max(peak_batches, st["batches"])
            if k:
                busy += now - tb
            elif done_submitting.is_set() and st["queued"] == 0 and st["resident"] == 0:
                break
            else:
                time.sleep(0.001)
        st = srv.stats()
        frames, chunks, psteps, rejected = (st["frames"], st["chunks"],
                                            st["particle_steps"], st["rejected"])
        from types import SimpleNamespace
        done = [SimpleNamespace(rid=i, t_arrival=arrivals[i][0], t_done=finished[i])
                for i in finished]
        host_s = {"server_steps": busy, "chunks": chunks}
    else:
        while not (done_submitting.is_set() and not srv.queue and not srv.resident):
            tb = time.perf_counter()
            srv.admit()
            if srv.resident:
                peak_resident = max(peak_resident, len(srv.resident))
                peak_particles = max(peak_particles, sum(r.n for r in srv.resident))
                peak_batches = max(peak_batches, sum(1 for sh in srv.shards if sh.resident))
                srv.step_chunk()
                busy += time.perf_counter() - tb
            else:
                time.sleep(0.001)
        frames, chunks, psteps, rejected = (srv.frames, srv.chunks, srv.particle_steps,
                                            len(srv.rejected))
        done = srv.done
        host_s = {"step_and_sync": srv.t_step, "repack": srv.t_repack,
                  "readback": srv.t_readback, "chunks": chunks}
    makespan = time.perf_counter() - t0
    clk = clocks.stop()
    th.join()
    srv.close()
    if errors:
        raise errors[0]
    makespan = R.max(makespan)
    served = R.sum(psteps) / makespan
    lat = S.latency_stats(done)
    offered = sum(sp["nx"] * sp["ny"] * sp["nz"] * k for _, sp, k in trace)
    loop = fifo_loop_executed(g, W, S, trace, local, args.graph_frames)
    loop["value"] = R.sum(loop["value"])
    return {
        "value": served, "unit": "particle-steps/s",
        "workload": f"{len(trace)} requests over {duration:g} s (Poisson 50/s), "
                    f"N log-uniform [8192, 1048576], K uniform [50, 500]",
        "latency": lat, "requests": len(done), "frames": frames, "chunks": chunks,
        "offered_particle_steps": offered, "makespan_s": makespan,
        "server_busy_s": busy, "ms_per_frame": busy * 1e3 / max(frames, 1),
        "host_s": host_s, "rejected": rejected,
        "budget_gb": args.budget_gb, "capacity_particles": cap[0],
        "capacity_cells": cap[1], "chunk_frames": args.chunk,
        "max_batches": max_batches, "peak_batches": peak_batches,
        "server": "native gsph_server_*" if native else "Python SceneServer",
        "peak_resident_scenes": peak_resident, "peak_resident_particles": peak_particles,
        "per_scene_fifo_loop": loop,
        "speedup_vs_loop": served / loop["value"],
        "p50_vs_loop": lat["p50_ms"] / loop["latency"]["p50_ms"],
        "p99_vs_loop": lat["p99_ms"] / loop["latency"]["p99_ms"],
        "clocks": clk,
        "gpu_launches": LAUNCHES_PER_FRAME * frames + chunks,
    }


def run_served(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    R = Ranks(ws)
    g = load_pkg()
    W = load_workloads()
    S = load_serve()
    rec = served_record(g, W, S, args, R, rank, local, args.duration)
    line = {
        "metric": "served aggregate particle-steps/s with p50/p99 completion latency",
        "value": rec["value"], "unit": "particle-steps/s", "n_gpus": ws,
        "steps": rec["frames"], "warmup": args.warmup, "ms_per_step": rec["ms_per_frame"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded Poisson trace of jittered dam-break columns, "
                "lattices built on arrival",
        "config": {"workload": "served: " + rec["workload"],
                   **{k: rec[k] for k in ("budget_gb", "capacity_particles",
                                          "capacity_cells", "chunk_frames", "server",
                                          "max_batches")}},
        **{k: rec[k] for k in ("latency", "requests", "offered_particle_steps",
                               "makespan_s", "server_busy_s", "host_s", "rejected",
                               "peak_resident_scenes", "peak_resident_particles",
                               "peak_batches", "per_scene_fifo_loop", "speedup_vs_loop", "p50_vs_loop",
                               "p99_vs_loop", "clocks", "gpu_launches")},
    }
    if rank == 0:
        print(json.dumps(line))
    R.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the end-to-end loop (profiling runs)")
    ap.add_argument("--scene", default=SCENE)
    ap.add_argument("--workload", default="single", choices=["single", "batched", "served", "stress"])
    ap.add_argument("--scenes", type=int, default=256, help="batched: scene count")
    ap.add_argument("--graph-frames", type=int, default=10)
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched: keep the reference thresholds and default shapes")
    ap.add_argument("--duration", type=float, default=60.0, help="served: seconds of traffic")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="served: HBM state budget")
    ap.add_argument("--cap-particles", type=int, default=40_000_000,
                    help="served: particle capacity of the resident batch")
    ap.add_argument("--chunk", type=int, default=10, help="served: frames between admissions")
    ap.add_argument("--max-batches", type=int, default=0,
                    help="served: batches the server may open (0: as many as the budget "
                         "holds at their capacity)")
    ap.add_argument("--server", default="native", choices=["native", "python"],
                    help="served: the C++ server (gsph_server_*) or the Python SceneServer")
    ap.add_argument("--no-batched", action="store_true",
                    help="single: leave the batched sub-record out of the line")
    ap.add_argument("--no-served", action="store_true",
                    help="single: leave the served sub-record out of the line")
    ap.add_argument("--batched-frames", type=int, default=100,
                    help="single: timed frames of the batched sub-record")
    ap.add_argument("--batched-graph-frames", type=int, default=100,
                    help="single: frames per CUDA graph in the batched sub-record")
    ap.add_argument("--served-duration", type=float, default=10.0,
                    help="single: seconds of arrivals in the served sub-record")
    ap.add_argument("--stress-side", type=int, default=256, help="stress: column side")
    ap.add_argument("--restart-frames", type=int, default=2000,
                    help="stress: frames before the snapshot")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    if args.workload == "batched":
        return run_batched(args, ws, rank, local)
    if args.workload == "served":
        return run_served(args, ws, rank, local)

    import torch
    torch.cuda.set_device(local)
    dist = Ranks(ws)
    g = load_pkg()
    if args.workload == "stress":
        sysm, workload, cpu_state = prepare_stress(g, args, local)
    else:
        sysm = g.HybridSystem(g.scene_path(args.scene), device=local)
        workload = WORKLOAD if args.scene == SCENE else args.scene
        s = g.load_scene(g.scene_path(args.scene))
        p = g.params_init(s)
        cpu_state = (p, g.lattice(s, p), None, None,
                     "FP64 frame(s) of the full {n}-particle scene")
    capture_key = (f"stress_{args.stress_side}" if args.workload == "stress"
                   else Path(args.scene).stem)
    line = measure_scene(g, sysm, args, ws, rank, local, dist, workload, cpu_state,
                         capture_key)
    # the batched and served forms of the same metric, on the same GPU(s)
    extra = {}
    if args.workload == "single":
        W = load_workloads()
        if not args.no_batched:
            extra["batched"] = batched_record(g, W, args, dist, rank, local,
                                              args.batched_frames, args.batched_graph_frames)
        if not args.no_served:
            extra["served"] = served_record(g, W, load_serve(), args, dist, rank, local,
                                            args.served_duration)
    if line is not None:
        line.update(extra)
        if extra:
            line["gpu_launches_sub_records"] = {k: v["gpu_launches"] for k, v in extra.items()}
        print(json.dumps(line))
    dist.close()
    return 0


def prepare_stress(g, args, local):
    """256^3 = 16,777,216-particle column with the 262,144-particle scene's
    physics and proportions (box 10.24 x 5.12 x 5.12 m, 512 x 256 x 256
    cells), stepped `restart_frames` frames from the lattice with CUDA graphs,
    saved to a snapshot and restarted from it."""
    import tempfile
    W = load_workloads()
    side = args.stress_side
    s = g.parse_scene(W.column_scene_text(side, side, side, seed=0))
    p = g.params_init(s)
    pos = g.lattice(s, p)
    t = time.perf_counter()
    with g.HybridSystem(params=p, positions=pos, device=local) as h:
        h.set_graph_mode(50)
        h.step(args.restart_frames)
        h.sync()
        gen_s = time.perf_counter() - t
        fd, path = tempfile.mkstemp(suffix=".gsnap")
        os.close(fd)
        h.save_snapshot(path)
    del pos
    try:
        sysm = g.load_snapshot(path, device=local)
    finally:
        os.remove(path)
    sysm.arrange()                 # the grid of the restarted state
    cnt = sysm.copy_out(g.FIELD_CELL_COUNT)
    occ = cnt[cnt > 0]
    workload = (f"stress: {side}^3 = {side ** 3:,} FP32 particles restarted from a snapshot "
                f"after {args.restart_frames} frames of the 262k dam-break physics "
                f"(generated in {gen_s:.1f} s); grid {tuple(p.grid_size)}, occupied cells "
                f"{len(occ):,}, occupancy mean {occ.mean():.2f}, max {int(occ.max())} "
                f"({occ.max() / occ.mean():.2f}x mean)")
    sample = min(2_000_000, sysm.n)
    spos = sysm.copy_out(g.FIELD_POSITION)[:sample].copy()
    svel = sysm.copy_out(g.FIELD_VELOCITY)[:sample].copy()
    sev = sysm.copy_out(g.FIELD_EVAL_VELOCITY)[:sample].copy()
    return sysm, workload, (p, spos, svel, sev,
                            "FP64 frame(s) of the first {n} particles (sorted order) of the "
                            "restarted state")


def measure_scene(g, sysm, args, ws, rank, local, dist, workload, cpu_state, capture_key):
    import torch
    n = sysm.n
    stream = torch.cuda.ExternalStream(sysm.stream(), device=torch.device("cuda", local))

    # frames run as CUDA graphs of `graph_frames` frames (the library's fastest
    # launch mode); the warm-up also captures the graph, so no capture falls in
    # the timed region
    sysm.set_graph_mode(args.graph_frames)
    sysm.step(max(args.warmup, 0))
    if args.graph_frames > 0:
        sysm.step(args.graph_frames)
    sysm.sync()

    clocks = ClockSampler(local)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev0.record(stream)
    sysm.step(args.steps)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed_ms = ev0.elapsed_time(ev1)
    # per-stage device times (events between the stages) on the frames right
    # after the timed ones, launched frame by frame
    sysm.set_stage_timing(True)
    sysm.step(max(10, min(args.steps, 50)))
    stages = sysm.stage_times()
    sysm.set_stage_timing(False)
    elapsed_ms = dist.max(elapsed_ms)
    sysm.sync()
    ms_per_step = elapsed_ms / max(args.steps, 1)
    value = ws * n * args.steps / (elapsed_ms / 1e3)

    # roofline of the dominant kernel (force or density)
    counts = sysm.copy_out(g.FIELD_CELL_COUNT)
    b_den, b_for = tile_bytes(counts, tuple(sysm.params.grid_size), n)
    # gsph_step fuses the integration into the force pass, which then also
    # reads the velocity and writes the new position, velocity and evaluated
    # velocity: 64 B per particle more than the force alone.
    fused = stages["integrate"] < 0.05 * stages["force"]
    if fused:
        b_for += 64 * n
    dom = "force" if stages["force"] >= stages["density"] else "density"
    b_dom = b_for if dom == "force" else b_den
    t_dom = stages[dom] / 1e3
    peak, peak_kind = measured_peak()
    achieved = b_dom / t_dom / 1e9 if t_dom > 0 else 0.0
    info = sysm.info()
    # the stage is one TRA and one SMS launch; name the one that does the work
    kernel = f"k_{dom}_" + ("sms" if info.tra_particles == 0 else "tra")
    traffic = ncu_traffic(kernel, capture_key)
    # both passes against the same cell-tile model (each stage = its TRA and
    # SMS launches back to back)
    per_stage = {}
    for st, b in (("density", b_den), ("force", b_for)):
        t_s = stages[st] / 1e3
        a = b / t_s / 1e9 if t_s > 0 else 0.0
        per_stage[st] = {"achieved": a, "frac": a / peak, "algorithmic_bytes": b,
                         "ms": stages[st]}
    if fused:
        per_stage["force"]["note"] = "integration fused into the force pass"

    # end to end through the public API: host-resident state, pinned buffers
    host = [torch.empty((n, 4), dtype=torch.float32, pin_memory=True) for _ in range(3)]
    fields = (g.FIELD_POSITION, g.FIELD_VELOCITY, g.FIELD_EVAL_VELOCITY)
    for h, f in zip(host, fields):
        sysm.copy_out_async(f, h.data_ptr(), h.numel() * 4)
    sysm.sync()
    e2e_steps = 0 if args.no_e2e else max(3, min(args.steps, 20))
    dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ptrs = [h.data_ptr() for h in host]
    for _ in range(e2e_steps):
        # upload pos/vel/ev from the pinned arrays, one frame, download them
        # back (gsph_step_host_async); each array's upload waits for its own
        # download from the previous frame
        sysm.step_host_async(1, *ptrs)
    sysm.sync()
    e2e_s = time.perf_counter() - t0
    e2e_s = dist.max(e2e_s)
    e2e_value = ws * n * e2e_steps / e2e_s if e2e_steps else None
    state_bytes = 3 * n * 16

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cp, cpos, cvel, cev, what = cpu_state
        rate, steps, cnt, thr = cpu_oracle_rate(cp, cpos, budget_s=12.0, max_steps=4,
                                                vel=cvel, ev=cev)
        cpu = {"value": rate, "unit": "particle-steps/s", "cores": thr, "kind": "port",
               "sample": f"{steps} " + what.format(n=cnt) +
                         " (C/OpenMP restatement of the reference step)"}
    sysm.close()
    if rank != 0:
        return None
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded jittered dam-break lattice generated on the host",
        "config": {"workload": workload, "particles": n,
                   "parallelism": f"{ws} independent replica(s)" if ws > 1 else "single GPU",
                   "l2": f"no flush: {n * 112 / 1e6:.0f} MB particle state per frame > 129 MB L2",
                   "timing": "CUDA events on the scene stream around K frames launched "
                             f"as CUDA graphs of {args.graph_frames} frames; stage times "
                             "from events between the stages of the frames that follow",
                   "graph_frames": args.graph_frames},
        "stages_ms": stages,
        "split": {"tra_particles": info.tra_particles, "sms_tasks": info.sms_tasks,
                  "occupied_cells": info.occupied_cells},
        "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "algorithmic_bytes": b_dom,
                     "traffic_source": (f"profiles/traffic_per_launch.txt, ncu capture of "
                                        f"{capture_key}") if traffic else
                                       "no ncu capture of this workload",
                     "fp32_pipe_frac": ncu_traffic(kernel, capture_key, "fma_pipe"),
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                     if peak_kind == "measured" else "fallback 6800 GB/s"},
        "roofline_stages": per_stage,
        "e2e": {"value": e2e_value, "unit": "particle-steps/s",
                "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes,
                "steps": e2e_steps,
                "method": "gsph_step_host_async(1 frame) per step on pinned host "
                          "pos/vel/ev; one sync after the last step"},
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": LAUNCHES_PER_FRAME * args.steps,
    }
    return line




if __name__ == "__main__":
    sys.exit(main())
