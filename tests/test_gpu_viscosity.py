"""Monaghan's artificial viscosity (GSPH_VISCOSITY_ARTIFICIAL) against the
FP64 oracle.

The benchmark configurations specify "artificial viscosity alpha = 0.02" with
c0 = 20 m/s; the reference has only Mueller's Laplacian viscosity
(src/solver/force_kernels.cu:378-435), which the parity runs use with alpha
mapped onto it. This optional mode replaces the Laplacian term in both force
passes (TRA and SMS) by Monaghan's term. Checked here on a sparse (all TRA),
a dense (all SMS) and a crowded mixed scene with random velocities, through
the stage entry points and through full frames, with the force bound of
test_gpu_parity.py.
"""
import numpy as np
import pytest

from gpu_helpers import dam_scene, dense_scene, shuffled

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-4
FORCE_SUM_TOL = 64 * 2.0 ** -24
ALPHA, C0 = 0.02, 20.0


def _crowded(gsph):
    _, p, pos = dam_scene(gsph, n_side=16, box=(0.8, 0.5, 0.5), seed=4)
    pos = pos.copy()
    pos[:, :3] = 0.1 + (pos[:, :3] - 0.1) * 0.4
    return None, p, pos


SCENES = {
    "sparse_tra": lambda g: dam_scene(g, n_side=16),
    "dense_sms": lambda g: dense_scene(g, n_side=24),
    "crowded_mixed": _crowded,
}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_artificial_viscosity_force_vs_fp64(gsph, oracle, cuda_device, name):
    _, p, pos = SCENES[name](gsph)
    pos = shuffled(pos)
    rng = np.random.default_rng(7)
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0.0, 0.5, (len(pos), 3))
    with gsph.HybridSystem(params=p, positions=pos, velocities=vel) as h:
        h.set_viscosity_model(gsph.VISCOSITY_ARTIFICIAL, ALPHA, C0)
        h.arrange()
        sv = h.copy_out(gsph.FIELD_VELOCITY)
        ev = h.copy_out(gsph.FIELD_EVAL_VELOCITY)
        ev[:, :3] = sv[:, :3]
        h.copy_in(gsph.FIELD_EVAL_VELOCITY, ev)
        h.density()
        h.force()
        spos = h.copy_out(gsph.FIELD_POSITION)
        sev = h.copy_out(gsph.FIELD_EVAL_VELOCITY)
        acc = h.copy_out(gsph.FIELD_ACCELERATION)[:, :3].astype(np.float64)
        ks = h.copy_out(gsph.FIELD_KEY)
        cs = h.copy_out(gsph.FIELD_CELL_START)
        info = h.info()
    ref, mag = oracle.force(spos, sev, ks, cs, p, with_mag=True, artificial=(ALPHA, C0))
    lap = oracle.force(spos, sev, ks, cs, p)
    fn = np.linalg.norm(ref, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fn ** 2))
    bound = FORCE_TOL * np.maximum(fn, floor) + FORCE_SUM_TOL * mag
    dev = np.linalg.norm(acc - ref, axis=1)
    assert np.all(dev <= bound), (name, (dev / bound).max())
    assert np.median(dev / np.maximum(fn, floor)) <= 1e-5
    # the mode changed the force: the Laplacian result is far outside the bound
    # (not in the crowded scene, whose ~10^13 pressure forces dwarf viscosity)
    if name != "crowded_mixed":
        assert np.median(np.linalg.norm(lap - ref, axis=1) / bound) > 10
    if name == "dense_sms":
        assert info.sms_tasks > 0
    if name == "sparse_tra":
        assert info.tra_particles == len(pos)
    if name == "crowded_mixed":
        assert info.sms_tasks > 0 and info.tra_particles > 0


def test_artificial_viscosity_in_full_frames(gsph, oracle, cuda_device):
    """Fused frames (force + integration in one pass, CUDA graphs) use the
    model too: one frame equals the stage sequence bit for bit, and switching
    back to the Laplacian model gives the default handle's bits."""
    _, p, pos = dam_scene(gsph, n_side=14, box=(0.6, 0.4, 0.4))
    fields = (gsph.FIELD_POSITION, gsph.FIELD_VELOCITY, gsph.FIELD_EVAL_VELOCITY)
    with gsph.HybridSystem(params=p, positions=pos) as h:
        h.set_viscosity_model(gsph.VISCOSITY_ARTIFICIAL, ALPHA, C0)
        h.set_graph_mode(3)
        h.step(6)
        fused = [h.copy_out(f) for f in fields]
    with gsph.HybridSystem(params=p, positions=pos) as h:
        h.set_viscosity_model(gsph.VISCOSITY_ARTIFICIAL, ALPHA, C0)
        for _ in range(6):
            h.arrange()
            h.density()
            h.force()
            h.advance()
        staged = [h.copy_out(f) for f in fields]
    for a, b in zip(fused, staged):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    with gsph.HybridSystem(params=p, positions=pos) as h:
        h.step(4)
        default = [h.copy_out(f) for f in fields]
    with gsph.HybridSystem(params=p, positions=pos) as h:
        h.set_viscosity_model(gsph.VISCOSITY_ARTIFICIAL, ALPHA, C0)
        h.set_viscosity_model(gsph.VISCOSITY_LAPLACIAN)
        h.step(4)
        back = [h.copy_out(f) for f in fields]
    for a, b in zip(default, back):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_viscosity_model_arguments(gsph, cuda_device):
    _, p, pos = dam_scene(gsph, n_side=6)
    with gsph.HybridSystem(params=p, positions=pos) as h:
        for model, a, c in ((2, 0.1, 1.0), (gsph.VISCOSITY_ARTIFICIAL, 0.0, 20.0),
                            (gsph.VISCOSITY_ARTIFICIAL, 0.1, -1.0),
                            (gsph.VISCOSITY_ARTIFICIAL, float("nan"), 1.0)):
            with pytest.raises(gsph.GsphError) as ei:
                h.set_viscosity_model(model, a, c)
            assert ei.value.status == gsph.ERR_INVALID_ARG
        h.step(2)
