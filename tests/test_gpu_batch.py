"""Batched step: every scene of a batch evolves exactly as it does alone.

gsph_batch_create steps several independent scenes with one launch per stage
(segmented sort over the concatenated cell space, one persistent work queue
for density and force). The sort order, the neighbour visiting order and the
arithmetic of each particle depend only on its own scene, so a scene's state
after K frames in the batch must be bit-identical to the same scene stepped
alone.
"""
import numpy as np
import pytest

from gpu_helpers import dam_scene, dense_scene, shuffled

pytestmark = pytest.mark.gpu


def _alone(gsph, p, pos, steps):
    with gsph.HybridSystem(params=p, positions=pos) as s:
        s.step(steps)
        return [s.copy_out(f) for f in (gsph.FIELD_POSITION, gsph.FIELD_VELOCITY,
                                        gsph.FIELD_EVAL_VELOCITY, gsph.FIELD_KEY)]


def _batch(gsph, scenes, steps, graph=False):
    with gsph.Batch(scenes) as b:
        b.set_graph_mode(graph)
        b.step(steps)
        out = []
        for k in range(len(scenes)):
            out.append([b.copy_out_scene(k, f) for f in (gsph.FIELD_POSITION,
                                                         gsph.FIELD_VELOCITY,
                                                         gsph.FIELD_EVAL_VELOCITY,
                                                         gsph.FIELD_KEY)])
        info = b.info()
    return out, info


def _same(a, b):
    return all(np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(a, b))


def test_sparse_batch_bit_identical_to_alone(gsph, cuda_device):
    rng = np.random.default_rng(0)
    scenes = []
    for k, (n_side, box) in enumerate([(10, (0.6, 0.4, 0.4)), (16, (0.8, 0.5, 0.5)),
                                       (7, (0.3, 0.3, 0.3)), (13, (1.0, 0.4, 0.6))]):
        s, p, pos = dam_scene(gsph, n_side=n_side, box=box, seed=k)
        scenes.append((p, shuffled(pos, seed=k)))
    steps = 12
    batched, info = _batch(gsph, scenes, steps)
    assert info.n_scenes == len(scenes)
    for (p, pos), got in zip(scenes, batched):
        assert _same(got, _alone(gsph, p, pos, steps))
    graphed, _ = _batch(gsph, scenes, steps, graph=True)
    for a, b in zip(batched, graphed):
        assert _same(a, b)
    assert rng is not None


def test_dense_batch_bit_identical_to_alone(gsph, cuda_device):
    scenes = []
    for k, n_side in enumerate([12, 20, 9]):
        s, p, pos = dense_scene(gsph, n_side=n_side, seed=10 + k)
        scenes.append((p, shuffled(pos, seed=k)))
    steps = 4
    batched, info = _batch(gsph, scenes, steps)
    assert info.sms_tasks > 0
    for (p, pos), got in zip(scenes, batched):
        assert _same(got, _alone(gsph, p, pos, steps))


def _alone_model(gsph, p, pos, steps, model):
    with gsph.HybridSystem(params=p, positions=pos) as s:
        s.set_viscosity_model(*model)
        s.step(steps)
        return [s.copy_out(f) for f in (gsph.FIELD_POSITION, gsph.FIELD_VELOCITY,
                                        gsph.FIELD_EVAL_VELOCITY, gsph.FIELD_KEY)]


def test_artificial_viscosity_batch_bit_identical_to_alone(gsph, cuda_device):
    """The optional Monaghan viscosity is a handle setting that the batch's
    force passes read like every other parameter: sparse scenes and a crowded
    one (TRA and SMS cells) in a batch evolve as each does alone, launched
    frame by frame and as CUDA graphs."""
    model = (gsph.VISCOSITY_ARTIFICIAL, 0.02, 20.0)
    scenes = []
    for k, (n_side, box) in enumerate([(10, (0.6, 0.4, 0.4)), (14, (0.8, 0.5, 0.5)),
                                       (8, (0.4, 0.4, 0.4))]):
        _, p, pos = dam_scene(gsph, n_side=n_side, box=box, seed=20 + k)
        scenes.append((p, shuffled(pos, seed=k)))
    crowd = scenes[1][1].copy()
    crowd[:, :3] = 0.1 + (crowd[:, :3] - 0.1) * 0.4
    scenes.append((scenes[1][0], crowd))
    steps = 6
    for graph in (False, True):
        with gsph.Batch(scenes) as b:
            b.set_viscosity_model(*model)
            b.set_graph_mode(3 if graph else 0)
            b.step(steps)
            got = [[b.copy_out_scene(k, f) for f in (gsph.FIELD_POSITION, gsph.FIELD_VELOCITY,
                                                     gsph.FIELD_EVAL_VELOCITY, gsph.FIELD_KEY)]
                   for k in range(len(scenes))]
            info = b.info()
        assert info.sms_tasks > 0 and info.tra_particles > 0
        for (p, pos), g in zip(scenes, got):
            assert _same(g, _alone_model(gsph, p, pos, steps, model))


def test_batch_past_the_row_prefetch_size_bit_identical_to_alone(gsph, cuda_device):
    """Four scenes in 2.25M-cell boxes: together their cell arrays (8 bytes a
    cell) pass 64 MB, so the batch's TRA density pass is the build that
    prefetches its rows' offsets, while each scene alone (18 MB) runs the
    other build. The bits must not change."""
    scenes = []
    for k, n_side in enumerate([10, 12, 8, 11]):
        _, p, pos = dam_scene(gsph, n_side=n_side, box=(3.0, 3.0, 2.0), seed=40 + k)
        scenes.append((p, shuffled(pos, seed=k)))
    cells = int(np.prod(list(scenes[0][0].grid_size)))
    assert cells * 8 < 64 << 20 < 4 * cells * 8
    steps = 5
    batched, info = _batch(gsph, scenes, steps)
    assert info.n_cells == 4 * cells
    for (p, pos), got in zip(scenes, batched):
        assert _same(got, _alone(gsph, p, pos, steps))


def test_batch_rejects_mixed_physics(gsph, cuda_device):
    _, p1, pos1 = dam_scene(gsph, n_side=6)
    _, p2, pos2 = dense_scene(gsph, n_side=6)
    with pytest.raises(gsph.GsphError) as ei:
        gsph.Batch([(p1, pos1), (p2, pos2)])
    assert ei.value.status == gsph.ERR_INVALID_ARG


def test_batch_rejects_key_space_overflow(gsph, cuda_device):
    """Cell keys are 32-bit micro keys (cells x 64 < 2^32): a batch whose
    scenes hold 2^26 cells or more together is refused before any device
    allocation, although each scene fits alone."""
    _, p, pos = dam_scene(gsph, n_side=4, box=(6.0, 6.0, 6.0))   # 300^3 cells
    cells = int(np.prod(list(p.grid_size)))
    assert cells < 2 ** 26 <= 3 * cells
    with gsph.Batch([(p, pos)]) as b:          # one scene fits
        assert b.info().n_cells == cells
    with pytest.raises(gsph.GsphError) as ei:
        gsph.Batch([(p, pos)] * 3)
    assert ei.value.status == gsph.ERR_CAPACITY


def test_batch_handles_empty_scene(gsph, cuda_device):
    _, p1, pos1 = dam_scene(gsph, n_side=8)
    _, p2, pos2 = dam_scene(gsph, n_side=9, box=(0.5, 0.4, 0.4))
    scenes = [(p1, pos1), (p2, pos2[:0]), (p2, pos2)]
    batched, _ = _batch(gsph, scenes, 5)
    assert len(batched[1][0]) == 0
    assert _same(batched[0], _alone(gsph, p1, pos1, 5))
    assert _same(batched[2], _alone(gsph, p2, pos2, 5))


def _load_serve(gsph):
    import importlib.util
    import sys
    name = "gsph_gb300.serve"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, gsph.PKG_DIR / "serve.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def test_served_results_identical_alone_and_in_the_mix(gsph, cuda_device):
    """Requests arrive while others are being stepped, are admitted between
    chunks, share the batched step and retire at different frames; each
    final state equals the scene stepped alone, bit for bit."""
    serve = _load_serve(gsph)
    specs = [(9, (0.5, 0.4, 0.4), 13, 0), (12, (0.7, 0.5, 0.5), 8, 3),
             (7, (0.3, 0.3, 0.4), 17, 3), (14, (0.8, 0.5, 0.5), 6, 9),
             (8, (0.4, 0.4, 0.4), 11, 14)]
    reqs = []
    for k, (n_side, box, steps, arrive) in enumerate(specs):
        _, p, pos = dam_scene(gsph, n_side=n_side, box=box, seed=20 + k)
        reqs.append((arrive, serve.Request(k, p, shuffled(pos, seed=k), steps, 0.0)))
    alone = {}
    for _, r in reqs:
        with gsph.HybridSystem(params=r.params, positions=r.pos) as s:
            s.step(r.steps)
            alone[r.rid] = (s.copy_out(gsph.FIELD_POSITION), s.copy_out(gsph.FIELD_VELOCITY))
    frame = [0]
    srv = serve.SceneServer(gsph, budget_bytes=1 << 34, capacity=(200000, 400000, 16),
                            chunk=4, clock=lambda: float(frame[0]))
    pending = sorted(reqs, key=lambda x: x[0])
    while pending or srv.queue or srv.resident:
        while pending and pending[0][0] <= frame[0]:
            srv.submit(pending.pop(0)[1])
        srv.admit()
        if srv.resident:
            before = srv.frames
            srv.step_chunk()
            frame[0] += srv.frames - before
        elif pending:
            frame[0] = pending[0][0]
    srv.close()
    assert len(srv.done) == len(reqs)
    for r in srv.done:
        pos, vel = alone[r.rid]
        assert np.array_equal(r.result["pos"].view(np.uint32), pos.view(np.uint32)), r.rid
        assert np.array_equal(r.result["vel"].view(np.uint32), vel.view(np.uint32)), r.rid
    # the mix really overlapped: some request waited for others and shared frames
    assert any(r.t_admit > r.t_arrival for r in srv.done) or srv.frames < sum(
        r.steps for r in srv.done)


def test_repack_rejects_capacity_overflow(gsph, cuda_device):
    _, p, pos = dam_scene(gsph, n_side=8)
    with gsph.Batch([(p, pos)], capacity=(len(pos) + 10, p.numc * 2, 2)) as b:
        with pytest.raises(gsph.GsphError) as ei:
            b.repack([0], [(p, pos)])
        assert ei.value.status == gsph.ERR_CAPACITY
        b.step(2)                       # the batch is unchanged and usable
        assert b.num_scenes == 1
        b.repack([], [])                # no scene left: stepping is a no-op
        b.step(3)
        b.repack([], [(p, pos)])
        b.step(1)
        assert b.num_scenes == 1
