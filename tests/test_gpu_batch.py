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


def test_batch_rejects_mixed_physics(gsph, cuda_device):
    _, p1, pos1 = dam_scene(gsph, n_side=6)
    _, p2, pos2 = dense_scene(gsph, n_side=6)
    with pytest.raises(gsph.GsphError) as ei:
        gsph.Batch([(p1, pos1), (p2, pos2)])
    assert ei.value.status == gsph.ERR_INVALID_ARG


def test_batch_handles_empty_scene(gsph, cuda_device):
    _, p1, pos1 = dam_scene(gsph, n_side=8)
    _, p2, pos2 = dam_scene(gsph, n_side=9, box=(0.5, 0.4, 0.4))
    scenes = [(p1, pos1), (p2, pos2[:0]), (p2, pos2)]
    batched, _ = _batch(gsph, scenes, 5)
    assert len(batched[1][0]) == 0
    assert _same(batched[0], _alone(gsph, p1, pos1, 5))
    assert _same(batched[2], _alone(gsph, p2, pos2, 5))
