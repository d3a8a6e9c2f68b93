"""Coincident and nearly coincident particles against the FP64 oracle.

Every density and force loop of the reference leaves out the pairs with
r^2 < kFloatSmall = 1e-12 (core/cuda_math.cuh:14; density_kernels.cu:172 and
:289, force_kernels.cu:407 and :539): the particle itself and any particle on
top of it. The density passes here test kFloatSmall <= r^2 <= h^2 with one
unsigned compare on r^2 - kFloatSmall (its roundings differ from the
two-compare form). These tests plant, next to interior particles of a TRA
scene and of an all-SMS scene, exact duplicates, a triple, and partners at
about 4e-7 m (r^2 ~ 1.6e-13: left out) and 3e-6 m (r^2 ~ 9e-12: counted, with
a weight close to the particle's own), and check density (<= 1e-5 relative)
and force (the condition-aware bound of test_gpu_parity.py) on every particle,
and the TRA neighbour counts, against the oracle's FP64 sums with the same
rule.
"""
import numpy as np
import pytest

from gpu_helpers import dam_scene, dense_scene

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
FORCE_TOL = 1e-4
FORCE_SUM_TOL = 64 * 2.0 ** -24
BAND = 1e-6
SEPARATIONS = (0.0, 4e-7, 3e-6)   # r^2 = 0, ~1.6e-13, ~9e-12


def plant(pos, per_kind, seed):
    """Adds per_kind partners at each separation (and one triple) next to
    distinct particles picked at random."""
    rng = np.random.default_rng(seed)
    picks = rng.choice(len(pos), size=per_kind * len(SEPARATIONS) + 1, replace=False)
    extra = []
    for k, s in enumerate(SEPARATIONS):
        for i in picks[k * per_kind:(k + 1) * per_kind]:
            u = rng.normal(size=3)
            u /= np.linalg.norm(u)
            q = pos[i].copy()
            q[:3] = (pos[i, :3].astype(np.float64) + s * u).astype(np.float32)
            extra.append(q)
    t = picks[-1]
    extra += [pos[t].copy(), pos[t].copy()]   # three particles on one point
    return np.concatenate([pos, np.array(extra, np.float32)])


def neighbour_band(spos, h2):
    """Per particle, the FP64 count of partners with 1e-12 <= r^2 <= h^2,
    taken over the band h^2 (1 -+ 1e-6)."""
    from scipy.spatial import cKDTree
    x = spos[:, :3].astype(np.float64)
    tree = cKDTree(x)
    lo = tree.query_ball_point(x, np.sqrt(h2 * (1 - BAND)), return_length=True)
    hi = tree.query_ball_point(x, np.sqrt(h2 * (1 + BAND)), return_length=True)
    near = tree.query_ball_point(x, 1e-6, return_length=True)   # r^2 < 1e-12
    return lo - near, hi - near


SCENES = {
    "sparse_tra": lambda g: dam_scene(g, n_side=16),
    "dense_sms": lambda g: dense_scene(g, n_side=20),
}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_coincident_pairs_vs_fp64(gsph, oracle, cuda_device, name):
    _, p, pos = SCENES[name](gsph)
    rng = np.random.default_rng(3)
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0.0, 0.3, (len(pos), 3))
    planted = plant(pos, per_kind=40, seed=5)
    vel = np.concatenate([vel, np.zeros((len(planted) - len(pos), 4), np.float32)])
    order = np.random.default_rng(17).permutation(len(planted))
    with gsph.HybridSystem(params=p, positions=planted[order], velocities=vel[order]) as h:
        h.arrange()
        h.copy_in(gsph.FIELD_EVAL_VELOCITY, h.copy_out(gsph.FIELD_VELOCITY))
        h.density()
        cnt = h.copy_out(gsph.FIELD_NEIGHBOR_COUNT)
        h.force()
        spos = h.copy_out(gsph.FIELD_POSITION)
        sev = h.copy_out(gsph.FIELD_EVAL_VELOCITY)
        acc = h.copy_out(gsph.FIELD_ACCELERATION)[:, :3].astype(np.float64)
        ks = h.copy_out(gsph.FIELD_KEY)
        cs = h.copy_out(gsph.FIELD_CELL_START)
        info = h.info()
    if name == "sparse_tra":
        assert info.tra_particles == len(planted)
    else:
        assert info.sms_tasks > 0

    rho, _ = oracle.density(spos, ks, cs, p)
    e_rho = np.abs(1.0 / spos[:, 3].astype(np.float64) - rho) / rho
    assert e_rho.max() <= RHO_TOL, e_rho.max()
    fo, mag = oracle.force(spos, sev, ks, cs, p, with_mag=True)
    fn = np.linalg.norm(fo, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fn ** 2))
    bound = FORCE_TOL * np.maximum(fn, floor) + FORCE_SUM_TOL * mag
    dev = np.linalg.norm(acc - fo, axis=1)
    assert np.all(dev <= bound), (dev / bound).max()

    # the planted pairs are in the sorted state, on both sides of 1e-12
    x = spos[:, :3].astype(np.float64)
    from scipy.spatial import cKDTree
    tree = cKDTree(x)
    pairs = tree.query_pairs(1e-5, output_type="ndarray")
    d2 = ((x[pairs[:, 0]] - x[pairs[:, 1]]) ** 2).sum(axis=1)
    assert (d2 < 1e-12).sum() >= 40 + 3 and ((d2 > 4e-12) & (d2 < 2e-11)).sum() >= 35
    tra = cnt >= 0
    if tra.any():
        lo, hi = neighbour_band(spos, float(np.float32(p.kernel_2)))
        bad = tra & ((cnt < lo) | (cnt > hi))
        assert not bad.any(), (cnt[bad][:5], lo[bad][:5], hi[bad][:5])
