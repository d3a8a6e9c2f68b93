"""Continuous-batching scene server over the batched step.

Requests (a scene's initial state and a number of frames) wait in a FIFO
queue and are admitted between chunks of frames while the device state of all
resident scenes fits the memory budget. Resident scenes stay on the device
and are stepped together (one launch per stage for all of them); a scene that
has done its frames is retired and its final state copied to the host. Every
chunk stops at the earliest completion, so each scene is stepped exactly its
requested number of frames, and since a scene's evolution inside a batch is
bit-identical to its evolution alone, the result does not depend on the mix.
"""
from __future__ import annotations

import collections
import time

import numpy as np


# Device bytes a scene holds in a batch: particle state (two buffer sets),
# force, sort and split workspace, neighbour masks and the occupied-cell lists
# (bounded by the particle count) per particle; cell offsets, slab words and
# group offsets per cell.
BYTES_PER_PARTICLE = 221
BYTES_PER_CELL = 44


def scene_bytes(n_particles: int, n_cells: int) -> int:
    return BYTES_PER_PARTICLE * n_particles + BYTES_PER_CELL * n_cells


class Request:
    __slots__ = ("rid", "params", "pos", "steps", "t_arrival", "t_admit", "t_done",
                 "remaining", "result", "n", "cells")

    def __init__(self, rid, params, pos, steps, t_arrival):
        self.rid = rid
        self.params = params
        self.pos = pos
        self.steps = int(steps)
        self.t_arrival = t_arrival
        self.t_admit = None
        self.t_done = None
        self.remaining = int(steps)
        self.result = None
        self.n = len(pos)
        self.cells = params.numc


class SceneServer:
    def __init__(self, g, budget_bytes: int, capacity=None, chunk: int = 10,
                 device: int = 0, keep_results: bool = True, clock=time.perf_counter):
        """capacity = (particles, cells, scenes) reserved on the device; the
        budget additionally bounds admission."""
        self.g = g
        self.budget = int(budget_bytes)
        self.capacity = capacity
        self.chunk = int(chunk)
        self.device = device
        self.keep_results = keep_results
        self.clock = clock
        self.queue = collections.deque()
        self.resident = []            # Requests, in batch order
        self.batch = None
        self.done = []
        self.rejected = []            # requests that cannot fit even alone
        self.frames = 0
        self.chunks = 0
        self.particle_steps = 0
        self.t_step = 0.0             # host seconds in step + sync
        self.t_repack = 0.0           # host seconds in batch creation / repack
        self.t_readback = 0.0         # host seconds reading finished results

    # ------------------------------------------------------------- intake --
    def submit(self, req: Request) -> None:
        self.queue.append(req)

    def _live(self):
        return [r for r in self.resident if r.remaining > 0]

    def _fits(self, reqs) -> bool:
        n = sum(r.n for r in reqs)
        c = sum(r.cells for r in reqs)
        if sum(scene_bytes(r.n, r.cells) for r in reqs) > self.budget:
            return False
        if self.capacity is not None:
            pc, cc, sc = self.capacity
            if n > pc or c > cc or len(reqs) > sc:
                return False
        return True

    def admit(self, allow_new: bool = True) -> int:
        """Admit queued requests (FIFO) that fit beside the live scenes and
        drop the retired ones, with one repack; returns how many were admitted."""
        live = self._live()
        new = []
        while allow_new:
            while self.queue and self._fits(live + new + [self.queue[0]]):
                new.append(self.queue.popleft())
            # a head that cannot fit even alone would block the queue forever
            if self.queue and not self._fits([self.queue[0]]):
                self.rejected.append(self.queue.popleft())
                continue
            break
        if not new and len(live) == len(self.resident):
            return 0
        now = self.clock()
        for r in new:
            r.t_admit = now
        t = time.perf_counter()
        scenes = [(r.params, r.pos) for r in new]
        keep = [i for i, r in enumerate(self.resident) if r.remaining > 0]
        if self.batch is None:
            if scenes:
                self.batch = self.g.Batch(scenes, device=self.device, capacity=self.capacity)
                self.batch.set_graph_mode(0)
        else:
            self.batch.repack(keep, scenes)
        self.t_repack += time.perf_counter() - t
        self.resident = live + new
        for r in new:
            r.pos = None          # the state now lives on the device
        return len(new)

    # --------------------------------------------------------------- work --
    def step_chunk(self):
        """Step all live scenes up to the earliest completion (at most `chunk`
        frames) and read back the finished ones' results. Finished scenes
        leave the batch at the next admit() (or here, before stepping)."""
        if len(self._live()) != len(self.resident):
            self.admit(allow_new=False)
        if not self.resident:
            return []
        k = min(self.chunk, min(r.remaining for r in self.resident))
        t = time.perf_counter()
        self.batch.step(k)
        self.batch.sync()
        self.t_step += time.perf_counter() - t
        self.frames += k
        self.chunks += 1
        self.particle_steps += sum(r.n for r in self.resident) * k
        for r in self.resident:
            r.remaining -= k
        out = []
        t = time.perf_counter()
        for i, r in enumerate(self.resident):
            if r.remaining:
                continue
            if self.keep_results:
                r.result = {
                    "pos": self.batch.copy_out_scene(i, self.g.FIELD_POSITION),
                    "vel": self.batch.copy_out_scene(i, self.g.FIELD_VELOCITY),
                }
            else:
                self.batch.copy_out_scene(i, self.g.FIELD_POSITION)   # result read-back
            r.t_done = self.clock()
            out.append(r)
        self.t_readback += time.perf_counter() - t
        self.done += out
        return out

    def close(self):
        if self.batch is not None:
            self.batch.close()
            self.batch = None


def latency_stats(reqs):
    lat = np.array([r.t_done - r.t_arrival for r in reqs])
    if len(lat) == 0:
        return {"p50_ms": None, "p99_ms": None, "mean_ms": None}
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3)}
