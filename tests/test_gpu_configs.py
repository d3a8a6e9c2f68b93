"""Parity on the benchmark scenes themselves, through the C ABI.

The 262,144-particle dam break (64^3, seed 0, box 2.56 x 1.28 x 1.28 m,
128 x 64 x 64 cells) and the 3,944,312-particle one that the benchmark times
(158^3, seed 0, box 4.74 x 3.16 x 1.68 m, 237 x 159 x 84 cells) each run one
frame through this library and through the reference's own kernels (the
harness in oracle/refharness, which replays HybridSystem::tick(),
src/simulation/sph_hybrid_system.cpp:253-339, with the reference's unmodified
kernels) on the same input state, twice: the lattice at rest, and the state
the library reaches after some hundred frames (moving fluid, some cells on
the SMS path). Compared, matched by particle identity:

  grid     sorted keys, coarse cell offsets and counts, every occupied micro
           cell's start and count, the canonical permutation
           (src/grid/sph_arrangement.cu:1352-1395): bit-exact
  split    block_req, middle, task count, every task field, and the TRA and
           SMS particle sets of the compact index per cell (:87-107,
           :885-1022, src/io/gpu_model.cu:137-181): bit-exact
  density  |d rho| / rho <= 1e-5 against the reference's kernels and against
           the FP64 oracle, on every particle
  force    within the condition-aware bound of test_gpu_parity.py against
           the FP64 oracle (every particle) and against the reference's
           kernels (twice that bound: both sides round)
  advance  positions within 1e-6 of the box, velocities within 1e-5 of the
           largest speed, against the reference's integrator.
"""
import json

import numpy as np
import pytest

import oracle.refharness as ref
from golden_util import canonical_perm, source_ids

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
FORCE_TOL = 1e-4
FORCE_SUM_TOL = 64 * 2.0 ** -24
POS_TOL = 1e-6

CONFIGS = {
    # scene file, frames the library steps before the moving-state comparison
    "dam_262k": ("dam_break_262k.json", 1500),
    "dam_3_94m": ("dam_break_3_94m.json", 300),
}


def _library_frame(gsph, p, pos, vel, ev):
    out = {}
    with gsph.HybridSystem(params=p, positions=pos, velocities=vel) as s:
        s.copy_in(gsph.FIELD_EVAL_VELOCITY, ev)
        s.arrange()
        for name, f in (("key", gsph.FIELD_KEY), ("perm", gsph.FIELD_PERMUTATION),
                        ("cs", gsph.FIELD_CELL_START), ("cnt", gsph.FIELD_CELL_COUNT),
                        ("req", gsph.FIELD_BLOCK_REQ), ("split", gsph.FIELD_SPLIT),
                        ("compact", gsph.FIELD_COMPACT_INDEX), ("tasks", gsph.FIELD_TASKS),
                        ("spos", gsph.FIELD_POSITION)):
            out[name] = s.copy_out(f)
        s.density()
        out["dpos"] = s.copy_out(gsph.FIELD_POSITION)
        out["dev"] = s.copy_out(gsph.FIELD_EVAL_VELOCITY)
        s.force()
        out["acc"] = s.copy_out(gsph.FIELD_ACCELERATION)[:, :3].astype(np.float64)
        s.advance()
        out["fpos"] = s.copy_out(gsph.FIELD_POSITION)
        out["fvel"] = s.copy_out(gsph.FIELD_VELOCITY)
    return out


def _moving_state(gsph, p, pos, frames):
    with gsph.HybridSystem(params=p, positions=pos) as s:
        s.set_graph_mode(50)
        s.step(frames)
        s.sync()
        return (s.copy_out(gsph.FIELD_POSITION), s.copy_out(gsph.FIELD_VELOCITY),
                s.copy_out(gsph.FIELD_EVAL_VELOCITY))


def _compare(gsph, oracle, p, pos, vel, ev, label):
    n = len(pos)
    L = _library_frame(gsph, p, pos, vel, ev)
    R = ref.run_tick(p, pos, vel, ev)
    report = {"case": label, "particles": n}

    # ---- grid: bit-exact
    ref_keys = R["hash"].view(np.uint32)
    key = L["key"]
    assert np.array_equal(key, ref_keys), "sorted keys"
    cs = L["cs"]
    assert np.array_equal(cs[:-1], R["cell_offset"]), "cell offsets"
    assert np.array_equal(L["cnt"], R["cell_nump"]), "cell counts"
    mk, mstart, mcount = np.unique(key, return_index=True, return_counts=True)
    assert int(R["micro_total"]) == n
    assert np.array_equal(mk.astype(np.int64), R["micro_index"]), "occupied micro cells"
    assert np.array_equal(mstart, R["micro_start"]), "micro cell starts"
    assert np.array_equal(mcount, R["micro_count"]), "micro cell counts"
    ref_ids = source_ids(R["sorted_pos"], pos)
    perm = L["perm"]
    assert np.array_equal(perm, canonical_perm(ref_keys, ref_ids)), "permutation"

    # ---- split and tasks: bit-exact
    assert np.array_equal(L["req"], R["block_req"]), "block_req"
    T = int(R["task_count"])
    ref_mid = int(R["middle"])
    middle = n if ref_mid < 0 else ref_mid
    assert L["split"][0] == middle and L["split"][1] == T, (L["split"], middle, T)
    for f in ("is_same", "paired_bounds", "cellid", "cell_pos", "p_offset", "xxi", "xxx",
              "yyi", "yyy", "zzi", "zzz", "cell_begin", "cell_particle_count"):
        assert np.array_equal(L["tasks"][f][:T], R["tasks"][f][:T]), f
    # compact index: the same source particles on each side of the split, cell by
    # cell (the reference's order inside a cell's TRA bucket comes from atomics)
    cell_of_src = np.empty(n, np.int64)
    cell_of_src[ref_ids] = (ref_keys >> 6).astype(np.int64)
    for part_l, part_r in ((L["compact"][:middle], R["index"][:middle]),
                           (L["compact"][middle:], R["index"][middle:])):
        src_l = perm[part_l]
        src_r = ref_ids[part_r]
        cl, cr = cell_of_src[src_l], cell_of_src[src_r]
        assert np.all(np.diff(cl) >= 0) and np.all(np.diff(cr) >= 0), "compact order by cell"
        assert np.array_equal(src_l[np.lexsort((src_l, cl))], src_r[np.lexsort((src_r, cr))])

    # ---- physics per particle identity
    where_ref = np.empty(n, np.int64)
    where_ref[ref_ids] = np.arange(n)
    r = where_ref[perm]
    rho = 1.0 / L["dpos"][:, 3].astype(np.float64)
    rho_ref = 1.0 / R["density_pos"][r, 3].astype(np.float64)
    orho, _ = oracle.density(L["spos"], key, cs, p)
    e_ref = np.abs(rho - rho_ref) / rho_ref
    e_64 = np.abs(rho - orho) / orho
    report["density_vs_reference"] = float(e_ref.max())
    report["density_vs_fp64"] = float(e_64.max())
    assert e_ref.max() <= RHO_TOL and e_64.max() <= RHO_TOL

    fo, mag = oracle.force(L["dpos"], L["dev"], key, cs, p, with_mag=True)
    fn = np.linalg.norm(fo, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fn ** 2))
    bound = FORCE_TOL * np.maximum(fn, floor) + FORCE_SUM_TOL * mag
    d64 = np.linalg.norm(L["acc"] - fo, axis=1)
    dref = np.linalg.norm(L["acc"] - R["force_acc"][r].astype(np.float64), axis=1)
    report["force_vs_fp64_max_over_bound"] = float((d64 / bound).max())
    report["force_vs_reference_max_over_bound"] = float((dref / (2 * bound)).max())
    report["force_vs_fp64_median_rel"] = float(np.median(d64 / np.maximum(fn, floor)))
    assert np.all(d64 <= bound) and np.all(dref <= 2 * bound)
    assert report["force_vs_fp64_median_rel"] <= 1e-5

    box = max(p.world_size)
    dp = np.abs(L["fpos"][:, :3] - R["final_pos"][r, :3]).max()
    vs = max(np.abs(R["final_vel"]).max(), 1e-3)
    dv = np.abs(L["fvel"][:, :3] - R["final_vel"][r]).max()
    report["position_vs_reference_over_box"] = float(dp / box)
    report["velocity_vs_reference_over_max_speed"] = float(dv / vs)
    report["sms_tasks"] = T
    report["tra_particles"] = middle
    print("\n" + json.dumps(report))
    assert dp <= POS_TOL * box
    assert dv <= 1e-5 * vs


@pytest.mark.skipif(not ref.available(), reason="reference harness not built")
@pytest.mark.parametrize("config", sorted(CONFIGS))
def test_benchmark_scene_frame_matches_reference(gsph, oracle, cuda_device, config):
    scene_file, frames = CONFIGS[config]
    s = gsph.load_scene(gsph.scene_path(scene_file))
    p = gsph.params_init(s)
    pos = gsph.lattice(s, p)
    zero = np.zeros_like(pos)
    _compare(gsph, oracle, p, pos, zero, zero, f"{config} lattice at rest")
    mpos, mvel, mev = _moving_state(gsph, p, pos, frames)
    _compare(gsph, oracle, p, mpos, mvel, mev, f"{config} after {frames} frames")


def test_3_94m_grid_bit_exact_vs_oracle(gsph, oracle, cuda_device):
    """The benchmark scene's grid and split against the CPU oracle (no
    reference harness needed): keys, permutation, offsets, block_req, compact
    index and tasks bit-exact."""
    s = gsph.load_scene(gsph.scene_path("dam_break_3_94m.json"))
    p = gsph.params_init(s)
    pos = gsph.lattice(s, p)
    assert len(pos) == 3_944_312
    with gsph.HybridSystem(params=p, positions=pos) as h:
        h.arrange()
        key = h.copy_out(gsph.FIELD_KEY)
        perm = h.copy_out(gsph.FIELD_PERMUTATION)
        cs = h.copy_out(gsph.FIELD_CELL_START)
        req = h.copy_out(gsph.FIELD_BLOCK_REQ)
        compact = h.copy_out(gsph.FIELD_COMPACT_INDEX)
        split = h.copy_out(gsph.FIELD_SPLIT)
    ks, operm, ocs, bad = oracle.sort(pos, p)
    assert not bad
    assert np.array_equal(key, ks) and np.array_equal(perm, operm) and np.array_equal(cs, ocs)
    oreq = oracle.block_req(cs, p)
    assert np.array_equal(req, oreq)
    ocompact, middle = oracle.split(cs, oreq, p)
    assert split[0] == middle and split[1] == int(oreq.sum())
    assert np.array_equal(compact, ocompact)
