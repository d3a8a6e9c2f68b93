"""Large uneven-occupancy stress: a 256^3 = 16,777,216-particle dam-break
column (the 262,144-particle scene's physics and proportions: box 4x the
column width long, 2x its height and depth, 512 x 256 x 256 cells) is stepped
2,000 frames from the lattice, saved, restarted from the snapshot, and one
frame's density, pressure and force are compared with the FP64 oracle on a
seeded 1M-particle subset. The errors are printed per quantity; the bounds
are the parity bounds of the small scenes.
"""
import importlib.util
import sys

import numpy as np
import pytest

from conftest import PKG_DIR

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
FORCE_TOL = 1e-4
FORCE_SUM_TOL = 64 * 2.0 ** -24
P_ULPS = 8 * 2.0 ** -24     # pressure: rounding of (x^7 - 1) B in FP32
SIDE = 256
FRAMES = 2000
SUBSET = 1_000_000


def _workloads():
    name = "gsph_gb300.workloads"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, PKG_DIR / "workloads.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def test_stress_16m_restart_vs_fp64(gsph, oracle, cuda_device, tmp_path):
    W = _workloads()
    s = gsph.parse_scene(W.column_scene_text(SIDE, SIDE, SIDE, seed=0))
    p = gsph.params_init(s)
    pos = gsph.lattice(s, p)
    n = len(pos)
    assert n == SIDE ** 3
    snap = tmp_path / "stress.gsnap"
    with gsph.HybridSystem(params=p, positions=pos) as h:
        h.set_graph_mode(50)
        h.step(FRAMES)
        h.save_snapshot(snap)
    del pos
    with gsph.load_snapshot(snap) as h:
        assert h.info().frames == FRAMES
        h.arrange()
        cnt = h.copy_out(gsph.FIELD_CELL_COUNT)
        h.density()
        h.force()
        spos = h.copy_out(gsph.FIELD_POSITION)
        sev = h.copy_out(gsph.FIELD_EVAL_VELOCITY)
        acc = h.copy_out(gsph.FIELD_ACCELERATION)[:, :3].astype(np.float64)
        ks = h.copy_out(gsph.FIELD_KEY)
        cs = h.copy_out(gsph.FIELD_CELL_START)
        info = h.info()
    snap.unlink()
    occ = cnt[cnt > 0]
    idx = np.sort(np.random.default_rng(0).choice(n, SUBSET, replace=False))
    rho, pr = oracle.density(spos, ks, cs, p)
    gpu_rho = 1.0 / spos[idx, 3].astype(np.float64)
    rho_err = np.abs(gpu_rho - rho[idx]) / rho[idx]
    ref, mag = oracle.force(spos, sev, ks, cs, p, with_mag=True)
    ref, mag = ref[idx], mag[idx]
    fn = np.linalg.norm(ref, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fn ** 2))
    dev = np.linalg.norm(acc[idx] - ref, axis=1)
    f_rel = dev / np.maximum(fn, floor)
    f_bound = FORCE_TOL * np.maximum(fn, floor) + FORCE_SUM_TOL * mag
    B = float(p.gas_constant)
    p_bound = (7.0 * B * (rho[idx] / float(p.rest_density)) ** 7 * RHO_TOL
               + P_ULPS * (B + np.abs(pr[idx])))
    p_err = np.abs(sev[idx, 3] - pr[idx])
    print(f"\nstress 16.8M after {FRAMES} frames + restart: occupied cells {len(occ)}, "
          f"occupancy mean {occ.mean():.2f} max {occ.max()} ({occ.max() / occ.mean():.2f}x mean), "
          f"TRA particles {info.tra_particles}, SMS tasks {info.sms_tasks}\n"
          f"  density  rel err: max {rho_err.max():.3e} median {np.median(rho_err):.3e}\n"
          f"  pressure abs err: max {p_err.max():.3e} Pa (max/bound {(p_err / p_bound).max():.3f})\n"
          f"  force    rel err: max {f_rel.max():.3e} median {np.median(f_rel):.3e} "
          f"(max/bound {(dev / f_bound).max():.3f})")
    assert rho_err.max() <= RHO_TOL
    assert np.all(p_err <= p_bound)
    assert np.all(dev <= f_bound)
    assert np.median(f_rel) <= 1e-5
