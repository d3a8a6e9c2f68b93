"""Neighbour sets of the TRA pass on positions built to sit on the edges of
its candidate pruning.

Each TRA neighbour row keeps the micro-x slabs of the left cell from the
particle's own micro-x up and of the right cell up to it (the reference's rule,
kernel_common.cuh:69-112), and the density pass records the neighbours it
finds as bit masks that the force pass walks. Here particles sit on micro slab
and cell boundaries (exactly, and one FP32 ulp to either side), and pairs are
planted at distances h (1 + d) for small positive and negative d across cell
faces, edges and corners. For every TRA particle the number of neighbours the
density pass found (GSPH_FIELD_NEIGHBOR_COUNT) must lie between the number of
particles with d^2 <= h^2 (1 - 1e-6) and with d^2 <= h^2 (1 + 1e-6), computed
in FP64 from the same FP32 positions (the FP32 cut-off test differs from FP64
by a few units in the last place); density and force, the latter from the
recorded masks, then match the oracle within the parity bounds.
"""
import numpy as np
import pytest

from gpu_helpers import dam_scene, shuffled

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
FORCE_TOL = 1e-4
FORCE_SUM_TOL = 64 * 2.0 ** -24
BAND = 1e-6
LO, HI = 0.05, 0.45          # fluid sub-box (m); cell size 0.02


def boundary_positions(p, seed=3):
    """Random positions (8 per cell on average) with a third of the
    coordinates moved onto micro-slab boundaries (exactly, or one FP32 ulp
    below or above), plus pairs planted at distance h (1 + d) along face,
    edge and corner directions."""
    rng = np.random.default_rng(seed)
    rat = np.float32(4.0) * np.float32(p.inv_cell_size)
    n = int(8 * ((HI - LO) / p.cell_size) ** 3)
    pos = rng.uniform(LO, HI, size=(n, 3)).astype(np.float32)
    snap = rng.random((n, 3)) < 1.0 / 3.0
    k = np.floor(pos.astype(np.float64) * float(rat)).astype(np.float32)
    on = (k / rat).astype(np.float32)
    nudge = rng.integers(-1, 2, size=(n, 3))
    on = np.where(nudge < 0, np.nextafter(on, np.float32(0)), on)
    on = np.where(nudge > 0, np.nextafter(on, np.float32(1)), on)
    pos = np.where(snap, on, pos).astype(np.float32)

    h = float(p.kernel)
    dirs = []
    for v in [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1),
              (1, 1, 1), (1, -1, 0), (1, 0, -1), (1, -1, -1), (2, 1, 0), (3, 1, 1)]:
        a = np.array(v, np.float64)
        dirs.append(a / np.linalg.norm(a))
    deltas = [-3e-4, -1e-4, -2e-5, -1e-6, 0.0, 1e-6, 2e-5, 1e-4, 3e-4]
    m = 4000
    base = pos[rng.choice(n, m, replace=False)].astype(np.float64)
    d = np.array(dirs)[rng.integers(0, len(dirs), m)]
    d *= np.where(rng.random((m, 1)) < 0.5, -1.0, 1.0)
    dist = h * (1.0 + np.array(deltas)[rng.integers(0, len(deltas), m)])
    partner = base + d * dist[:, None]
    keep = np.all((partner > LO) & (partner < HI), axis=1)
    pos = np.concatenate([pos, partner[keep].astype(np.float32)])
    out = np.zeros((len(pos), 4), np.float32)
    out[:, :3] = pos
    return out


def band_counts(spos, h2):
    from scipy.spatial import cKDTree
    x = spos[:, :3].astype(np.float64)
    tree = cKDTree(x)
    lo = tree.query_ball_point(x, np.sqrt(h2 * (1 - BAND)), return_length=True)
    hi = tree.query_ball_point(x, np.sqrt(h2 * (1 + BAND)), return_length=True)
    # the cut-off test skips d^2 < 1e-12 (the particle itself and duplicates)
    same = tree.query_ball_point(x, 1e-6, return_length=True)
    return lo - same, hi - same


def test_tra_neighbor_sets_on_pruning_edges(gsph, oracle, cuda_device):
    _, p, _ = dam_scene(gsph, n_side=16)
    pos = shuffled(boundary_positions(p))
    with gsph.HybridSystem(params=p, positions=pos) as h:
        h.arrange()
        h.density()
        cnt = h.copy_out(gsph.FIELD_NEIGHBOR_COUNT)
        h.force()
        spos = h.copy_out(gsph.FIELD_POSITION)
        sev = h.copy_out(gsph.FIELD_EVAL_VELOCITY)
        acc = h.copy_out(gsph.FIELD_ACCELERATION)[:, :3].astype(np.float64)
        ks = h.copy_out(gsph.FIELD_KEY)
        cs = h.copy_out(gsph.FIELD_CELL_START)
    tra = cnt >= 0
    assert tra.mean() > 0.5, "the scene must run mostly on the TRA path"
    lo, hi = band_counts(spos, float(np.float32(p.kernel_2)))
    bad = tra & ((cnt < lo) | (cnt > hi))
    assert not bad.any(), (
        f"{int(bad.sum())} TRA particles with a neighbour count outside "
        f"[{lo[bad][:5]}, {hi[bad][:5]}]: {cnt[bad][:5]}")

    rho, _ = oracle.density(spos, ks, cs, p)
    gpu_rho = 1.0 / spos[:, 3].astype(np.float64)
    assert (np.abs(gpu_rho - rho) / rho).max() <= RHO_TOL
    ref, mag = oracle.force(spos, sev, ks, cs, p, with_mag=True)
    fn = np.linalg.norm(ref, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fn ** 2))
    dev = np.linalg.norm(acc - ref, axis=1)
    assert np.all(dev <= FORCE_TOL * np.maximum(fn, floor) + FORCE_SUM_TOL * mag)


def test_long_rows_fall_back_to_the_candidate_scan(gsph, oracle, cuda_device):
    """A lone TRA particle whose diagonal neighbour cells are crowded: its
    (dy, dz) = (-1, -1) row holds more than 32 candidates, so the density
    pass records no masks for it (neighbour count -1) and the force pass scans
    its candidates with the cut-off test. Density and force match the FP64
    oracle."""
    _, p, _ = dam_scene(gsph, n_side=16)
    rng = np.random.default_rng(21)
    cs_ = float(p.cell_size)
    lone = np.array([[10.25, 10.25, 10.25], [14.6, 14.3, 14.4]]) * cs_
    crowd = []
    for base in ([9, 9, 9], [13, 13, 13]):
        for dx in range(3):
            c = np.array(base, np.float64) + [dx, 0, 0]
            crowd.append((c + rng.uniform(0.02, 0.98, (40, 3))) * cs_)
    xyz = np.concatenate([lone] + crowd).astype(np.float32)
    pos = np.zeros((len(xyz), 4), np.float32)
    pos[:, :3] = xyz
    with gsph.HybridSystem(params=p, positions=shuffled(pos)) as h:
        h.arrange()
        h.density()
        cnt = h.copy_out(gsph.FIELD_NEIGHBOR_COUNT)
        h.force()
        spos = h.copy_out(gsph.FIELD_POSITION)
        sev = h.copy_out(gsph.FIELD_EVAL_VELOCITY)
        acc = h.copy_out(gsph.FIELD_ACCELERATION)[:, :3].astype(np.float64)
        ks = h.copy_out(gsph.FIELD_KEY)
        cs = h.copy_out(gsph.FIELD_CELL_START)
        split = h.copy_out(gsph.FIELD_SPLIT)
    is_lone = np.zeros(len(spos), bool)
    for q in lone.astype(np.float32):
        is_lone |= np.all(spos[:, :3] == q, axis=1)
    assert is_lone.sum() == 2
    assert split[0] >= 2 and split[1] > 0         # TRA and SMS particles both
    assert np.all(cnt[is_lone] == -1)
    lo, _ = band_counts(spos, float(np.float32(p.kernel_2)))
    assert np.all(lo[is_lone] > 0)                # the lone particles interact

    rho, _ = oracle.density(spos, ks, cs, p)
    gpu_rho = 1.0 / spos[:, 3].astype(np.float64)
    assert (np.abs(gpu_rho - rho) / rho).max() <= RHO_TOL
    ref, mag = oracle.force(spos, sev, ks, cs, p, with_mag=True)
    fn = np.linalg.norm(ref, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fn ** 2))
    dev = np.linalg.norm(acc - ref, axis=1)
    assert np.all(dev <= FORCE_TOL * np.maximum(fn, floor) + FORCE_SUM_TOL * mag)


@pytest.mark.parametrize("per_cell", [8, 12, 16, 150])
def test_random_mixed_split_vs_fp64(gsph, oracle, cuda_device, per_cell):
    """Uniform random positions at 8 / 12 / 16 / 150 particles per cell: the
    performance model sends from a few to all cells to SMS tasks and the rest
    to TRA, with TRA rows both shorter and longer than 32 candidates. Density
    and force match the FP64 oracle within the parity bounds."""
    _, p, _ = dam_scene(gsph, n_side=16)
    rng = np.random.default_rng(per_cell)
    lo, hi = 0.06, 0.26                           # 10 cells a side
    n = int(per_cell * ((hi - lo) / p.cell_size) ** 3)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(lo, hi, (n, 3))
    with gsph.HybridSystem(params=p, positions=pos) as h:
        h.arrange()
        split = h.copy_out(gsph.FIELD_SPLIT)
        h.density()
        h.force()
        spos = h.copy_out(gsph.FIELD_POSITION)
        sev = h.copy_out(gsph.FIELD_EVAL_VELOCITY)
        acc = h.copy_out(gsph.FIELD_ACCELERATION)[:, :3].astype(np.float64)
        ks = h.copy_out(gsph.FIELD_KEY)
        cs = h.copy_out(gsph.FIELD_CELL_START)
    assert split[1] > 0, "some cells must go to SMS tasks"
    if per_cell <= 16:
        assert split[0] > 0, "some particles must stay on TRA"
    rho, _ = oracle.density(spos, ks, cs, p)
    gpu_rho = 1.0 / spos[:, 3].astype(np.float64)
    assert (np.abs(gpu_rho - rho) / rho).max() <= RHO_TOL
    ref, mag = oracle.force(spos, sev, ks, cs, p, with_mag=True)
    fn = np.linalg.norm(ref, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fn ** 2))
    dev = np.linalg.norm(acc - ref, axis=1)
    assert np.all(dev <= FORCE_TOL * np.maximum(fn, floor) + FORCE_SUM_TOL * mag)
