"""Host logic of the scene server, on a fake batch (no GPU).

The fake records every call the server makes (create, repack, step, read
back) and keeps per-scene frame counters the way the device batch keeps the
scenes' state, so the tests check admission order, the budget and capacity
limits, that every request is stepped exactly its K frames, and that retired
scenes leave the batch in order.
"""
import importlib.util
import sys

import pytest

from conftest import PKG_DIR


def _serve():
    name = "gsph_gb300.serve"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, PKG_DIR / "serve.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


class FakeParams:
    def __init__(self, numc):
        self.numc = numc


class FakeBatch:
    log = []

    def __init__(self, scenes, device=0, capacity=None):
        self.frames = [0 for _ in scenes]
        self.ids = [id(s[1]) for s in scenes]
        FakeBatch.log.append(("create", len(scenes)))

    def set_graph_mode(self, frames):
        pass

    def repack(self, keep, add_scenes=()):
        assert list(keep) == sorted(keep)
        self.frames = [self.frames[i] for i in keep] + [0 for _ in add_scenes]
        FakeBatch.log.append(("repack", len(keep), len(add_scenes)))

    def step(self, k):
        self.frames = [f + k for f in self.frames]

    def sync(self):
        pass

    def copy_out_scene(self, i, field):
        return self.frames[i]

    def close(self):
        pass


class FakeG:
    Batch = FakeBatch
    FIELD_POSITION = 0
    FIELD_VELOCITY = 1


def _req(S, rid, n, k, cells=None, t=0.0):
    return S.Request(rid, FakeParams(cells if cells is not None else 2 * n),
                     [0] * n, k, t)


def test_every_request_gets_exactly_its_frames():
    S = _serve()
    FakeBatch.log = []
    srv = S.SceneServer(FakeG, budget_bytes=1 << 40, chunk=7, clock=lambda: 0.0)
    ks = [13, 5, 29, 8, 8, 21, 1]
    for i, k in enumerate(ks):
        srv.submit(_req(S, i, 100 + i, k))
        if i % 3 == 2:                  # arrivals interleaved with chunks
            srv.admit()
            srv.step_chunk()
    while srv.queue or srv.resident:
        srv.admit()
        srv.step_chunk()
    assert sorted(r.rid for r in srv.done) == list(range(len(ks)))
    for r in srv.done:
        assert r.result["pos"] == r.steps          # the fake counts frames
    assert srv.particle_steps == sum((100 + i) * k for i, k in enumerate(ks))


def test_budget_and_capacity_bound_admission_fifo():
    S = _serve()
    per = S.scene_bytes(1000, 2000)
    srv = S.SceneServer(FakeG, budget_bytes=2 * per, capacity=(10**9, 10**9, 8),
                        chunk=100, clock=lambda: 0.0)
    for i in range(4):
        srv.submit(_req(S, i, 1000, 10 + i))
    assert srv.admit() == 2
    assert [r.rid for r in srv.resident] == [0, 1]
    srv.step_chunk()                         # request 0 retires after 10 frames
    assert [r.rid for r in srv.done] == [0]
    assert srv.admit() == 1                  # FIFO: request 2 is next
    assert [r.rid for r in srv.resident] == [1, 2]
    srv = S.SceneServer(FakeG, budget_bytes=1 << 40, capacity=(2500, 10**9, 8),
                        chunk=100, clock=lambda: 0.0)
    for i in range(3):
        srv.submit(_req(S, i, 1000, 5))
    assert srv.admit() == 2                  # particle capacity binds


def test_request_larger_than_capacity_is_rejected_not_stuck():
    S = _serve()
    srv = S.SceneServer(FakeG, budget_bytes=1 << 40, capacity=(500, 10**9, 8),
                        chunk=10, clock=lambda: 0.0)
    srv.submit(_req(S, 0, 1000, 5))
    srv.submit(_req(S, 1, 100, 5))
    assert srv.admit() == 1
    assert [r.rid for r in srv.rejected] == [0]
    srv.step_chunk()
    assert [r.rid for r in srv.done] == [1]


def test_latency_stats():
    S = _serve()
    rs = []
    for i in range(100):
        r = _req(S, i, 10, 1, t=0.0)
        r.t_done = (i + 1) * 1e-3
        rs.append(r)
    st = S.latency_stats(rs)
    assert st["p50_ms"] == pytest.approx(50.5)
    assert st["p99_ms"] == pytest.approx(99.01)
    assert S.latency_stats([])["p99_ms"] is None


def test_batches_open_until_the_budget_binds():
    """With several batches allowed, a full batch (its cell capacity, the
    key space of one batch) does not stop admission: further batches open
    and the memory budget is what bounds the resident scenes, exactly."""
    S = _serve()
    FakeBatch.log = []
    per = S.scene_bytes(1000, 2000)
    # each batch holds 3 scenes' cells; the budget holds exactly 7 scenes
    srv = S.SceneServer(FakeG, budget_bytes=7 * per, capacity=(10**9, 6000, 64),
                        chunk=100, clock=lambda: 0.0, max_batches=10)
    for i in range(10):
        srv.submit(_req(S, i, 1000, 10 + i))
    assert srv.admit() == 7
    assert [len(sh.resident) for sh in srv.shards] == [3, 3, 1]
    assert sum(S.scene_bytes(r.n, r.cells) for r in srv.resident) == 7 * per
    assert [r.rid for r in srv.resident] == list(range(7))
    srv.step_chunk()                      # request 0 retires after 10 frames
    assert srv.admit() == 1               # FIFO: request 7 takes its place
    assert sorted(r.rid for r in srv.resident) == list(range(1, 8))
    while srv.queue or srv.resident:
        srv.admit()
        srv.step_chunk()
    assert sorted(r.rid for r in srv.done) == list(range(10))
    for r in srv.done:
        assert r.result["pos"] == r.steps
    # one batch only: the cell capacity binds first
    srv = S.SceneServer(FakeG, budget_bytes=7 * per, capacity=(10**9, 6000, 64),
                        chunk=100, clock=lambda: 0.0, max_batches=1)
    for i in range(10):
        srv.submit(_req(S, i, 1000, 10 + i))
    assert srv.admit() == 3
