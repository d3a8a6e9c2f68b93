"""Snapshot / restart: a handle restored from a snapshot continues the run bit
for bit (single scene and batch), and corrupted files are refused."""
import numpy as np
import pytest

from gpu_helpers import dam_scene, dense_scene, shuffled
from test_snapshot_format import write_snapshot

pytestmark = pytest.mark.gpu

FIELDS = ("FIELD_POSITION", "FIELD_VELOCITY", "FIELD_EVAL_VELOCITY")


def _state(gsph, h):
    return [h.copy_out(getattr(gsph, f)).view(np.uint32) for f in FIELDS]


def test_restart_continues_bit_for_bit(gsph, cuda_device, tmp_path):
    _, p, pos = dam_scene(gsph, n_side=14, seed=3)
    f = tmp_path / "one.gsnap"
    with gsph.HybridSystem(params=p, positions=shuffled(pos)) as a:
        a.step(7)
        a.save_snapshot(f)
        a.step(5)
        want = _state(gsph, a)
        frames = a.info().frames
    assert gsph.snapshot_info(f)["frames"] == 7
    with gsph.load_snapshot(f) as b:
        assert isinstance(b, gsph.HybridSystem) and not isinstance(b, gsph.Batch)
        b.step(5)
        got = _state(gsph, b)
        assert b.info().frames == frames
    for x, y in zip(want, got):
        assert np.array_equal(x, y)


def test_batch_restart_continues_bit_for_bit(gsph, cuda_device, tmp_path):
    scenes = []
    for k, n_side in enumerate([9, 13, 6]):
        _, p, pos = dam_scene(gsph, n_side=n_side, box=(0.6, 0.5, 0.4), seed=k)
        scenes.append((p, shuffled(pos, seed=k)))
    _, pd, posd = dense_scene(gsph, n_side=10)
    f = tmp_path / "batch.gsnap"
    with gsph.Batch(scenes) as a:
        a.step(4)
        a.save_snapshot(f)
        a.step(6)
        want = [[a.copy_out_scene(k, getattr(gsph, n)).view(np.uint32) for n in FIELDS]
                for k in range(len(scenes))]
    with gsph.load_snapshot(f) as b:
        assert isinstance(b, gsph.Batch) and b.num_scenes == len(scenes)
        b.step(6)
        for k in range(len(scenes)):
            got = [b.copy_out_scene(k, getattr(gsph, n)).view(np.uint32) for n in FIELDS]
            for x, y in zip(want[k], got):
                assert np.array_equal(x, y)
    # a dense (all-SMS) scene restarts the same way
    f2 = tmp_path / "dense.gsnap"
    with gsph.HybridSystem(params=pd, positions=posd) as a:
        a.step(2)
        a.save_snapshot(f2)
        a.step(2)
        want = _state(gsph, a)
    with gsph.load_snapshot(f2) as b:
        b.step(2)
        for x, y in zip(want, _state(gsph, b)):
            assert np.array_equal(x, y)


def test_hand_written_snapshot_loads_and_corruption_is_refused(gsph, cuda_device, tmp_path):
    _, p, pos = dam_scene(gsph, n_side=8)
    vel = np.zeros_like(pos)
    vel[:, 1] = -0.25
    f = tmp_path / "hand.gsnap"
    write_snapshot(f, [p], [(pos, vel, np.zeros_like(pos))], frames=3)
    with gsph.load_snapshot(f) as h:
        assert h.n == len(pos) and h.info().frames == 3
        assert np.array_equal(h.copy_out(gsph.FIELD_VELOCITY), vel)
        h.step(1)
    with gsph.HybridSystem(params=p, positions=pos, velocities=vel) as ref:
        ref.step(1)
        want = _state(gsph, ref)
    with gsph.load_snapshot(f) as h:
        h.step(1)
        for x, y in zip(want, _state(gsph, h)):
            assert np.array_equal(x, y)
    raw = bytearray(f.read_bytes())
    raw[-5] ^= 0x40
    f.write_bytes(bytes(raw))
    with pytest.raises(gsph.GsphError) as ei:
        gsph.load_snapshot(f)
    assert ei.value.status == gsph.ERR_PARSE
