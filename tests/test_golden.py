"""The CPU oracle pinned to the reference's own outputs (no GPU).

tests/golden/*.npz were recorded by tests/golden/make_golden.py: one frame of
the reference's own CUDA kernels (compiled unmodified from its sources and
driven by oracle/refharness) on four scenes — a sparse dam break (all TRA),
the reference's default-scene physics (all SMS), a mixed scene (TRA + SMS,
odd task count, every performance-model branch) and 32,768 particles of the
262,144-particle dam break (its physics and proportions at half the size). Integer stages must match
exactly (modulo the reference's run-to-run order inside a micro cell);
physics within the stated tolerances of the FP64 oracle.
"""
import numpy as np
import pytest

from golden_util import (SCENES, canonical_bucket_ids, canonical_perm, dense_micro, load,
                         source_ids, split_parts)

RHO_TOL = 1e-5
FORCE_TOL = 1e-4
FORCE_SUM_TOL = 64 * 2.0 ** -24
POS_TOL = 1e-6


@pytest.fixture(params=SCENES)
def fx(request, gsph):
    d, p = load(request.param, gsph.Params)
    return request.param, d, p


def test_grid_matches_reference(oracle, fx):
    name, d, p = fx
    ks, perm, cs, bad = oracle.sort(d["in_pos"], p)
    assert not bad
    ref_keys = d["hash"].view(np.uint32)
    assert np.array_equal(ks, ref_keys)                      # A2: sorted keys
    assert np.array_equal(cs[:-1], d["cell_offset"])         # A5: cellStart
    assert np.array_equal(np.diff(cs), d["cell_nump"])       # A5: cellCount
    assert np.array_equal(oracle.micro_start(ks, p), dense_micro(d))   # A3
    ids = source_ids(d["sorted_pos"], d["in_pos"])           # A4: reorder
    assert np.array_equal(canonical_perm(ref_keys, ids), perm)
    assert np.array_equal(d["sorted_vel"], d["in_vel"][ids, :3])
    assert np.array_equal(d["sorted_ev"], d["in_ev"][ids])


def test_split_and_tasks_match_reference(gsph, oracle, fx):
    name, d, p = fx
    n = len(d["in_pos"])
    ks, perm, cs, _ = oracle.sort(d["in_pos"], p)
    req = oracle.block_req(cs, p)
    assert np.array_equal(req, d["block_req"])                # A6
    compact, middle = oracle.split(cs, req, p)
    ref_mid = int(d["middle"])
    assert middle == (n if ref_mid < 0 else ref_mid)          # A7 (-1: no SMS)
    ids = source_ids(d["sorted_pos"], d["in_pos"])
    cell_of_id = np.empty(n, np.int64)
    cell_of_id[ids] = d["hash"].view(np.uint32) >> 6
    for ref_part, my_part in zip(split_parts(d["index"], ref_mid, n),
                                 split_parts(compact, middle, n)):
        a, ordered = canonical_bucket_ids(ids[ref_part], cell_of_id)
        b, _ = canonical_bucket_ids(perm[my_part], cell_of_id)
        assert ordered and np.array_equal(a, b)
    tasks = oracle.tasks(ks, cs, req, p, gsph.BLOCK_TASK_DTYPE)    # A8, A9
    ref = d["tasks"]
    T = int(d["task_count"])
    assert len(tasks) == len(ref) == T + (T & 1)
    for f in gsph.BLOCK_TASK_DTYPE.names:
        if f == "pad_":
            continue
        assert np.array_equal(tasks[f][:T], ref[f][:T]), f
    if T & 1:   # odd-tail descriptor: the fields the reference defines
        for f in ("is_same", "cellid", "cell_pos", "p_offset", "cell_begin",
                  "cell_particle_count"):
            assert np.array_equal(tasks[f][T], ref[f][T]), f
    if name == "mixed":
        assert T & 1 and 0 < middle < n


def test_density_matches_reference(oracle, fx):
    name, d, p = fx
    keys = d["hash"].view(np.uint32)
    cs = np.append(d["cell_offset"], len(keys)).astype(np.int32)
    rho, pr = oracle.density(d["sorted_pos"], keys, cs, p)
    ref_rho = 1.0 / d["density_pos"][:, 3].astype(np.float64)
    err = np.abs(ref_rho - rho) / rho
    assert err.max() <= RHO_TOL, (name, err.max())
    bound = 7.0 * float(p.gas_constant) * (rho / float(p.rest_density)) ** 7 * RHO_TOL + 1e-6
    assert np.all(np.abs(d["density_ev"][:, 3] - pr) <= bound)


def test_force_matches_reference(oracle, fx):
    name, d, p = fx
    keys = d["hash"].view(np.uint32)
    cs = np.append(d["cell_offset"], len(keys)).astype(np.int32)
    ref, mag = oracle.force(d["density_pos"], d["density_ev"], keys, cs, p, with_mag=True)
    fn = np.linalg.norm(ref, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fn ** 2))
    dev = np.linalg.norm(d["force_acc"].astype(np.float64) - ref, axis=1)
    assert np.all(dev <= FORCE_TOL * np.maximum(fn, floor) + FORCE_SUM_TOL * mag), name
    assert np.median(dev / np.maximum(fn, floor)) <= 1e-5


def test_integrate_matches_reference(oracle, fx):
    name, d, p = fx
    n = len(d["in_pos"])
    vel = np.zeros((n, 4))
    vel[:, :3] = d["sorted_vel"]
    P, V, E = oracle.integrate(d["density_pos"], vel, d["density_ev"], d["force_acc"], p)
    box = max(p.world_size)
    assert np.abs(d["final_pos"][:, :3] - P[:, :3]).max() <= POS_TOL * box
    vs = max(np.abs(V[:, :3]).max(), 1e-3)
    assert np.abs(d["final_vel"] - V[:, :3]).max() <= 1e-5 * vs
    assert np.abs(d["final_ev"][:, :3] - E[:, :3]).max() <= 1e-5 * vs
    assert np.array_equal(d["final_pos"][:, 3], d["density_pos"][:, 3])
