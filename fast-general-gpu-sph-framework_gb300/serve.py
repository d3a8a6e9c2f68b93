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


class Shard:
    """One batch and the requests resident in it, in batch order."""
    __slots__ = ("batch", "resident")

    def __init__(self):
        self.batch = None
        self.resident = []


class SceneServer:
    def __init__(self, g, budget_bytes: int, capacity=None, chunk: int = 10,
                 device: int = 0, keep_results: bool = True, clock=time.perf_counter,
                 max_batches: int = 1):
        """capacity = (particles, cells, scenes) reserved on the device for
        each batch; up to max_batches batches are opened as admissions need
        them (a batch's key space holds fewer than 2^26 cells), and the budget
        bounds the resident bytes of all batches together."""
        self.g = g
        self.budget = int(budget_bytes)
        self.capacity = capacity
        self.chunk = int(chunk)
        self.device = device
        self.keep_results = keep_results
        self.clock = clock
        self.max_batches = max(1, int(max_batches))
        self.queue = collections.deque()
        self.shards = []
        self.done = []
        self.rejected = []            # requests that cannot fit even alone
        self.frames = 0
        self.chunks = 0
        self.particle_steps = 0
        self.t_step = 0.0             # host seconds in step + sync
        self.t_repack = 0.0           # host seconds in batch creation / repack
        self.t_readback = 0.0         # host seconds reading finished results

    @property
    def resident(self):
        """Every resident request, batch by batch, each in batch order."""
        return [r for sh in self.shards for r in sh.resident]

    @property
    def batch(self):
        """The first batch (the only one unless max_batches > 1)."""
        return self.shards[0].batch if self.shards else None

    # ------------------------------------------------------------- intake --
    def submit(self, req: Request) -> None:
        self.queue.append(req)

    def _fits_shard(self, reqs) -> bool:
        if self.capacity is None:
            return True
        pc, cc, sc = self.capacity
        return (sum(r.n for r in reqs) <= pc and sum(r.cells for r in reqs) <= cc
                and len(reqs) <= sc)

    def _fits(self, reqs) -> bool:
        """One request set in one batch, within the budget."""
        return (sum(scene_bytes(r.n, r.cells) for r in reqs) <= self.budget
                and self._fits_shard(reqs))

    def admit(self, allow_new: bool = True) -> int:
        """Admit queued requests (FIFO): each goes to the first batch with room
        for it, or to a new batch while fewer than max_batches are open, while
        all resident bytes fit the budget; retired scenes leave their batches.
        One repack (or creation) per changed batch; returns how many were
        admitted."""
        live = [[r for r in sh.resident if r.remaining > 0] for sh in self.shards]
        new = [[] for _ in self.shards]
        used = sum(scene_bytes(r.n, r.cells) for sh in live for r in sh)
        count = 0
        while allow_new:
            while self.queue:
                h = self.queue[0]
                need = scene_bytes(h.n, h.cells)
                if used + need > self.budget:
                    break
                b = next((k for k in range(len(live))
                          if self._fits_shard(live[k] + new[k] + [h])), None)
                if b is None:
                    if len(live) >= self.max_batches or not self._fits_shard([h]):
                        break
                    live.append([])
                    new.append([])
                    self.shards.append(Shard())
                    b = len(live) - 1
                new[b].append(self.queue.popleft())
                used += need
                count += 1
            # a head that cannot fit even alone would block the queue forever
            if self.queue and not self._fits([self.queue[0]]):
                self.rejected.append(self.queue.popleft())
                continue
            break
        now = self.clock()
        for k, sh in enumerate(self.shards):
            if not new[k] and len(live[k]) == len(sh.resident):
                continue
            for r in new[k]:
                r.t_admit = now
            t = time.perf_counter()
            scenes = [(r.params, r.pos) for r in new[k]]
            keep = [i for i, r in enumerate(sh.resident) if r.remaining > 0]
            if sh.batch is None:
                if scenes:
                    sh.batch = self.g.Batch(scenes, device=self.device,
                                            capacity=self.capacity)
                    sh.batch.set_graph_mode(0)
            else:
                sh.batch.repack(keep, scenes)
            self.t_repack += time.perf_counter() - t
            sh.resident = live[k] + new[k]
            for r in new[k]:
                r.pos = None          # the state now lives on the device
        return count

    # --------------------------------------------------------------- work --
    def step_chunk(self):
        """Step all live scenes up to the earliest completion (at most `chunk`
        frames; every batch launched before any is waited for) and read back
        the finished ones' results. Finished scenes leave their batch at the
        next admit() (or here, before stepping)."""
        if any(r.remaining == 0 for r in self.resident):
            self.admit(allow_new=False)
        res = self.resident
        if not res:
            return []
        k = min(self.chunk, min(r.remaining for r in res))
        t = time.perf_counter()
        active = [sh for sh in self.shards if sh.resident]
        for sh in active:
            sh.batch.step(k)
        for sh in active:
            sh.batch.sync()
        self.t_step += time.perf_counter() - t
        self.frames += k
        self.chunks += 1
        self.particle_steps += sum(r.n for r in res) * k
        for r in res:
            r.remaining -= k
        out = []
        t = time.perf_counter()
        for sh in active:
            for i, r in enumerate(sh.resident):
                if r.remaining:
                    continue
                if self.keep_results:
                    r.result = {
                        "pos": sh.batch.copy_out_scene(i, self.g.FIELD_POSITION),
                        "vel": sh.batch.copy_out_scene(i, self.g.FIELD_VELOCITY),
                    }
                else:
                    sh.batch.copy_out_scene(i, self.g.FIELD_POSITION)   # read-back
                r.t_done = self.clock()
                out.append(r)
        self.t_readback += time.perf_counter() - t
        self.done += out
        return out

    def close(self):
        for sh in self.shards:
            if sh.batch is not None:
                sh.batch.close()
                sh.batch = None


def latency_stats(reqs):
    lat = np.array([r.t_done - r.t_arrival for r in reqs])
    if len(lat) == 0:
        return {"p50_ms": None, "p99_ms": None, "mean_ms": None}
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3)}
