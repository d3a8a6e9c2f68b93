"""Split thresholds, launch shapes and the autotuner.

The default tuning is the reference's performance model; other thresholds
move cells between the TRA and SMS paths, which changes roundings but not the
physics (density checked against FP64 with the parity bound). The autotuner
must leave the handle's state exactly as it found it.
"""
import numpy as np
import pytest

from gpu_helpers import dam_scene, dense_scene, shuffled

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
FIELDS = ("FIELD_POSITION", "FIELD_VELOCITY", "FIELD_EVAL_VELOCITY")


def _state(g, h):
    return [h.copy_out(getattr(g, f)).view(np.uint32).copy() for f in FIELDS]


def test_default_and_validation(gsph, cuda_device):
    _, p, pos = dam_scene(gsph, n_side=8)
    with gsph.HybridSystem(params=p, positions=pos) as h:
        t = h.get_tuning()
        assert t.as_dict() == gsph.tuning_default().as_dict()
        assert (t.sparse_total, t.sparse_self, t.mid_total) == (96, 15, 60)
        bad = gsph.tuning_default()
        bad.ctas_density_tra = 99
        with pytest.raises(gsph.GsphError) as ei:
            h.set_tuning(bad)
        assert ei.value.status == gsph.ERR_INVALID_ARG
        assert h.get_tuning().as_dict() == t.as_dict()


@pytest.mark.parametrize("thr", [(0x7FFFFFFF, 0x7FFFFFFF, 60), (0, 0, 0), (48, 8, 30)])
def test_thresholds_move_cells_and_keep_density(gsph, oracle, cuda_device, thr):
    """All TRA, all SMS, SMS-leaning: density within 1e-5 of FP64 each time."""
    _, p, pos = dense_scene(gsph, n_side=24)
    with gsph.HybridSystem(params=p, positions=shuffled(pos)) as h:
        t = gsph.tuning_default()
        t.sparse_total, t.sparse_self, t.mid_total = thr
        h.set_tuning(t)
        h.arrange()
        h.density()
        info = h.info()
        spos = h.copy_out(gsph.FIELD_POSITION)
        ks = h.copy_out(gsph.FIELD_KEY)
        cs = h.copy_out(gsph.FIELD_CELL_START)
    if thr[0] == 0x7FFFFFFF:
        assert info.tra_particles == len(pos) and info.sms_tasks == 0
    if thr == (0, 0, 0):
        assert info.tra_particles < len(pos) // 10
    rho, _ = oracle.density(spos, ks, cs, p)
    err = np.abs(1.0 / spos[:, 3].astype(np.float64) - rho) / rho
    assert err.max() <= RHO_TOL


def test_autotune_restores_state_and_installs_best(gsph, cuda_device):
    _, p, pos = dam_scene(gsph, n_side=20, box=(0.9, 0.5, 0.5))
    with gsph.HybridSystem(params=p, positions=shuffled(pos)) as h:
        h.step(3)
        before = _state(gsph, h)
        frames = h.info().frames
        best, ms = h.autotune(frames_per_trial=2)
        assert ms > 0
        assert h.get_tuning().as_dict() == best.as_dict()
        assert h.info().frames == frames
        for x, y in zip(before, _state(gsph, h)):
            assert np.array_equal(x, y)
        h.step(4)
        after_tuned = _state(gsph, h)
    # the same tuning set by hand gives the same continuation
    with gsph.HybridSystem(params=p, positions=shuffled(pos)) as h:
        h.step(3)
        h.set_tuning(best)
        h.step(4)
        for x, y in zip(after_tuned, _state(gsph, h)):
            assert np.array_equal(x, y)


def test_autotuner_caches_by_occupancy_histogram(gsph, cuda_device):
    _, p, pos = dam_scene(gsph, n_side=16, box=(0.8, 0.5, 0.5), seed=1)
    _, p2, pos2 = dam_scene(gsph, n_side=16, box=(0.8, 0.5, 0.5), seed=2)
    tuner = gsph.Autotuner(frames_per_trial=1)
    with gsph.HybridSystem(params=p, positions=pos) as h:
        t1, _, cached1 = tuner.tune(h)
    with gsph.HybridSystem(params=p2, positions=pos2) as h:
        t2, _, cached2 = tuner.tune(h)
        assert h.get_tuning().as_dict() == t1.as_dict()
    assert not cached1 and cached2 and t1.as_dict() == t2.as_dict()


def test_autotune_leaves_the_grid_to_be_rebuilt(gsph, oracle, cuda_device):
    """The trials sort their own states, so after autotune the grid arrays do
    not describe the restored state: stage calls need a new arrange (they are
    refused until then), and after it density matches the oracle."""
    _, p, pos = dam_scene(gsph, n_side=14, box=(0.6, 0.4, 0.4))
    with gsph.HybridSystem(params=p, positions=shuffled(pos)) as h:
        h.step(2)
        h.arrange()
        h.autotune(frames_per_trial=1)
        with pytest.raises(gsph.GsphError) as ei:
            h.density()
        assert ei.value.status == gsph.ERR_STATE
        h.arrange()
        h.density()
        spos = h.copy_out(gsph.FIELD_POSITION)
        ks = h.copy_out(gsph.FIELD_KEY)
        cs = h.copy_out(gsph.FIELD_CELL_START)
    rho, _ = oracle.density(spos, ks, cs, p)
    err = np.abs(1.0 / spos[:, 3].astype(np.float64) - rho) / rho
    assert err.max() <= RHO_TOL


@pytest.mark.parametrize("scene", ["sparse", "dense"])
def test_block_shapes_give_the_same_bits(gsph, cuda_device, scene):
    """Blocks of 4 warps (the same kernels built for that shape, twice the
    CTAs per SM) change only the scheduling: every particle's arithmetic and
    order are the same, so frames are bit-identical to blocks of 8 warps."""
    if scene == "sparse":
        _, p, pos = dam_scene(gsph, n_side=18, box=(0.8, 0.5, 0.5))
    else:
        _, p, pos = dense_scene(gsph, n_side=20)
    outs = []
    for warps, k in ((8, 1), (4, 2), (4, 1)):
        with gsph.HybridSystem(params=p, positions=shuffled(pos)) as h:
            t = gsph.tuning_default()
            t.warps_per_block = warps
            t.ctas_density_tra *= k
            t.ctas_density_sms *= k
            t.ctas_force_tra *= k
            t.ctas_force_sms *= k
            h.set_tuning(t)
            assert h.get_tuning().warps_per_block == warps
            h.step(4)
            outs.append(_state(gsph, h))
    for other in outs[1:]:
        for x, y in zip(outs[0], other):
            assert np.array_equal(x, y)


def test_block_shape_validation(gsph, cuda_device):
    _, p, pos = dam_scene(gsph, n_side=6)
    with gsph.HybridSystem(params=p, positions=pos) as h:
        for warps, dt in ((6, 6), (4, 13), (8, 7)):
            t = gsph.tuning_default()
            t.warps_per_block = warps
            t.ctas_density_tra = dt
            with pytest.raises(gsph.GsphError) as ei:
                h.set_tuning(t)
            assert ei.value.status == gsph.ERR_INVALID_ARG
        t = gsph.tuning_default()
        t.warps_per_block = 4
        t.ctas_density_tra = 12
        h.set_tuning(t)
        h.step(2)
