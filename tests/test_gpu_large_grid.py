"""A grid whose cell arrays exceed half of L2 (the TRA density pass then
prefetches its rows' cell offsets into L1 first) against the same fluid in a
small box, and against the FP64 oracle.

The fluid is the same block of particles in a 0.8 x 0.5 x 0.5 m box
(40 x 25 x 25 cells) and in a 5.12 x 5.12 x 3.2 m box (256 x 256 x 160 =
10,485,760 cells, 84 MB of cell offsets and slab words). A particle's
candidates are visited in the same order in both (rows in a fixed (dy, dz)
order, each row left to right along x, each cell in micro-key order), so
density and force must agree bit for bit, particle by particle; both must be
within the parity bounds of the FP64 oracle. The large box runs with blocks of
8 and of 4 warps (both builds of the prefetching pass).
"""
import numpy as np
import pytest

from gpu_helpers import dam_scene, shuffled

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
FORCE_TOL = 1e-4
FORCE_SUM_TOL = 64 * 2.0 ** -24


def _frame(gsph, p, pos, vel, warps=8):
    with gsph.HybridSystem(params=p, positions=pos, velocities=vel) as h:
        if warps != 8:
            t = gsph.tuning_default()
            t.warps_per_block = warps
            h.set_tuning(t)
        h.arrange()
        h.copy_in(gsph.FIELD_EVAL_VELOCITY, h.copy_out(gsph.FIELD_VELOCITY))
        h.density()
        h.force()
        out = {"perm": h.copy_out(gsph.FIELD_PERMUTATION),
               "pos": h.copy_out(gsph.FIELD_POSITION),
               "ev": h.copy_out(gsph.FIELD_EVAL_VELOCITY),
               "acc": h.copy_out(gsph.FIELD_ACCELERATION),
               "key": h.copy_out(gsph.FIELD_KEY),
               "cs": h.copy_out(gsph.FIELD_CELL_START)}
        info = h.info()
    return out, info


@pytest.mark.parametrize("warps", [8, 4])
def test_large_grid_matches_small_box_and_fp64(gsph, oracle, cuda_device, warps):
    _, p_small, pos = dam_scene(gsph, n_side=24, box=(0.8, 0.5, 0.5))
    _, p_large, pos_l = dam_scene(gsph, n_side=24, box=(5.12, 5.12, 3.2))
    assert np.array_equal(pos, pos_l)
    cells = int(np.prod(np.asarray(p_large.grid_size, np.int64)))
    assert cells * 8 > 64 << 20, cells
    assert int(np.prod(np.asarray(p_small.grid_size, np.int64))) * 8 < 64 << 20
    pos = shuffled(pos, seed=4)
    rng = np.random.default_rng(6)
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0.0, 0.3, (len(pos), 3))
    small, info_s = _frame(gsph, p_small, pos, vel)
    large, info_l = _frame(gsph, p_large, pos, vel, warps)
    assert info_s.tra_particles == len(pos) and info_l.tra_particles == len(pos)

    # per source particle: same bits
    for name in ("pos", "acc"):
        a = np.empty_like(small[name])
        b = np.empty_like(large[name])
        a[small["perm"]] = small[name]
        b[large["perm"]] = large[name]
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name

    run = large
    rho, _ = oracle.density(run["pos"], run["key"], run["cs"], p_large)
    e_rho = np.abs(1.0 / run["pos"][:, 3].astype(np.float64) - rho) / rho
    assert e_rho.max() <= RHO_TOL, e_rho.max()
    fo, mag = oracle.force(run["pos"], run["ev"], run["key"], run["cs"], p_large,
                           with_mag=True)
    fn = np.linalg.norm(fo, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fn ** 2))
    bound = FORCE_TOL * np.maximum(fn, floor) + FORCE_SUM_TOL * mag
    dev = np.linalg.norm(run["acc"][:, :3].astype(np.float64) - fo, axis=1)
    assert np.all(dev <= bound), (dev / bound).max()
