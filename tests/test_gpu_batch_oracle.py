"""The batched and served forms against the FP64 oracle, scene by scene.

A batch replaces the reference's process-global __constant__ parameters
(src/solver/device_context.cu:10) with a per-scene table (grid, cell base,
walls) that every kernel reads: the hash adds the scene's cell base, the
performance model, split and tasks find a cell's scene by binary search over
the cell bases, the density and force queues span all scenes. These tests
check that machinery against the oracle run on each scene's own arrays, not
only against the same library stepping the scene alone:

  * a batch of 16 uneven scenes (sparse dam-break columns of several sizes and
    boxes, all-SMS dense blocks, a mixed scene) after one arrange, density and
    force: each scene's keys, permutation and cell offsets bit-exact against
    the oracle's sort of that scene's input; density |d rho| / rho <= 1e-5
    and force within the condition-aware bound of test_gpu_parity.py against
    the FP64 oracle on the scene's own sorted arrays;
  * the same for two requests resident in a continuous-batching server in the
    middle of a trace, after admissions and retirements have repacked the
    batch (scenes at other particle and cell bases than when they arrived).
"""
import importlib.util
import sys

import numpy as np
import pytest

from gpu_helpers import dam_scene, dense_scene, shuffled

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
FORCE_TOL = 1e-4
FORCE_SUM_TOL = 64 * 2.0 ** -24


def _scene_checks(gsph, oracle, b, k, p, pos_before):
    """Scene k of batch b after arrange + density + force, against the
    oracle on the scene's own arrays; returns the worst errors."""
    key = b.copy_out_scene(k, gsph.FIELD_KEY)
    perm = b.copy_out_scene(k, gsph.FIELD_PERMUTATION)
    cs = b.copy_out_scene(k, gsph.FIELD_CELL_START)
    ks, operm, ocs, bad = oracle.sort(pos_before, p)
    assert not bad
    assert np.array_equal(key, ks), k
    assert np.array_equal(perm, operm), k
    assert np.array_equal(cs, ocs), k
    pos = b.copy_out_scene(k, gsph.FIELD_POSITION)
    ev = b.copy_out_scene(k, gsph.FIELD_EVAL_VELOCITY)
    acc = b.copy_out_scene(k, gsph.FIELD_ACCELERATION)[:, :3].astype(np.float64)
    assert np.array_equal(pos[:, :3], pos_before[perm, :3]), k
    rho, _ = oracle.density(pos, key, cs, p)
    e_rho = np.abs(1.0 / pos[:, 3].astype(np.float64) - rho) / rho
    assert e_rho.max() <= RHO_TOL, (k, e_rho.max())
    fo, mag = oracle.force(pos, ev, key, cs, p, with_mag=True)
    fn = np.linalg.norm(fo, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(fn ** 2))
    bound = FORCE_TOL * np.maximum(fn, floor) + FORCE_SUM_TOL * mag
    dev = np.linalg.norm(acc - fo, axis=1)
    assert np.all(dev <= bound), (k, (dev / bound).max())
    return float(e_rho.max()), float((dev / bound).max())


def _sms_block(p, cells_lo, cells, per_cell, seed):
    """Particles uniform in a cell-aligned block, `per_cell` per cell on
    average: every cell of the block takes the SMS path."""
    h = float(p.kernel)
    lo = np.asarray(cells_lo, np.float64) * h
    hi = lo + np.asarray(cells, np.float64) * h
    n = int(per_cell * np.prod(cells))
    rng = np.random.default_rng(seed)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(lo + 1e-3 * h, hi - 1e-3 * h, (n, 3))
    return pos


def _uneven_scenes(gsph):
    """16 scenes with one physics (h = 0.02): 12 sparse jittered columns of
    several sizes and boxes (TRA), one column crowded to ~23x its density
    (TRA and SMS cells side by side), three blocks of 60-100 particles per
    cell (all SMS)."""
    scenes = []
    sparse = [(6, (0.3, 0.3, 0.3)), (9, (0.5, 0.4, 0.4)), (11, (0.8, 0.3, 0.5)),
              (13, (0.6, 0.6, 0.4)), (16, (0.8, 0.5, 0.5)), (18, (1.2, 0.5, 0.5)),
              (7, (0.25, 0.4, 0.3)), (20, (0.9, 0.6, 0.6)), (10, (0.4, 0.8, 0.3)),
              (14, (0.7, 0.4, 0.7)), (8, (0.35, 0.35, 0.35)), (12, (0.5, 0.5, 0.5))]
    for k, (n_side, box) in enumerate(sparse):
        _, p, pos = dam_scene(gsph, n_side=n_side, box=box, seed=100 + k)
        scenes.append((p, shuffled(pos, seed=k)))
    p0, pos0 = scenes[4]
    crowd = pos0.copy()
    crowd[:, :3] = 0.1 + (crowd[:, :3] - 0.1) * 0.35
    scenes.append((p0, crowd))
    for k, (lo, cells, per) in enumerate([((5, 5, 5), (3, 3, 3), 60),
                                          ((4, 6, 5), (4, 2, 3), 100),
                                          ((6, 5, 4), (2, 2, 2), 80)]):
        scenes.append((p0, _sms_block(p0, lo, cells, per, seed=30 + k), "all_sms"))
    return scenes


def test_batch_of_16_uneven_scenes_vs_fp64(gsph, oracle, cuda_device):
    rng = np.random.default_rng(9)
    uneven = _uneven_scenes(gsph)
    dense = []   # the reference default physics (h = 0.03), a batch of its own
    for k, (n_side, seed) in enumerate([(10, 1), (14, 2), (8, 3)]):
        _, p, pos = dense_scene(gsph, n_side=n_side, seed=seed)
        dense.append((p, shuffled(pos, seed=50 + k)))
    for scenes, label in ((uneven, "16 uneven scenes"), (dense, "3 dense scenes")):
        plain = [(sc[0], sc[1]) for sc in scenes]
        vels = [np.concatenate([rng.normal(0, 0.2, (len(pos), 3)), np.zeros((len(pos), 1))],
                               axis=1).astype(np.float32) for _, pos in plain]
        with gsph.Batch([(p, pos, v) for (p, pos), v in zip(plain, vels)]) as b:
            b.arrange()
            # evaluated velocity = velocity, so the viscosity term is exercised
            b.copy_in(gsph.FIELD_EVAL_VELOCITY, b.copy_out(gsph.FIELD_VELOCITY))
            b.density()
            b.force()
            info = b.info()
            cnts = [b.copy_out_scene(k, gsph.FIELD_CELL_COUNT) for k in range(len(plain))]
            worst = [_scene_checks(gsph, oracle, b, k, p, pos)
                     for k, (p, pos) in enumerate(plain)]
        assert info.n_scenes == len(plain)
        assert info.sms_tasks > 0
        req = [oracle.block_req(np.concatenate([[0], np.cumsum(c)]).astype(np.int32), sc[0])
               for c, sc in zip(cnts, plain)]
        # the split over the whole batch is the sum of the scenes' own splits
        assert info.sms_tasks == sum(int(r.sum()) for r in req)
        for sc, c, r in zip(scenes, cnts, req):
            if len(sc) > 2:   # all-SMS scene: every occupied cell has SMS tasks
                assert np.array_equal(r > 0, c > 0)
        print(f"\n{label}: TRA particles {info.tra_particles}, SMS tasks {info.sms_tasks}, "
              f"density max rel err {max(w[0] for w in worst):.2e}, "
              f"force max dev/bound {max(w[1] for w in worst):.3f}")
    assert len(uneven) == 16


def _load_serve(gsph):
    name = "gsph_gb300.serve"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, gsph.PKG_DIR / "serve.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def test_served_requests_mid_trace_vs_fp64(gsph, oracle, cuda_device):
    serve = _load_serve(gsph)
    specs = [(9, (0.5, 0.4, 0.4), 12, 0), (12, (0.7, 0.5, 0.5), 40, 0),
             (7, (0.3, 0.3, 0.4), 8, 2), (14, (0.8, 0.5, 0.5), 40, 5),
             (8, (0.4, 0.4, 0.4), 6, 9), (10, (0.6, 0.4, 0.4), 40, 12)]
    reqs = []
    for k, (n_side, box, steps, arrive) in enumerate(specs):
        _, p, pos = dam_scene(gsph, n_side=n_side, box=box, seed=60 + k)
        reqs.append((arrive, serve.Request(k, p, shuffled(pos, seed=k), steps, 0.0)))
    frame = [0]
    srv = serve.SceneServer(gsph, budget_bytes=1 << 34, capacity=(200000, 400000, 8),
                            chunk=3, clock=lambda: float(frame[0]))
    pending = sorted(reqs, key=lambda x: x[0])
    # run the trace until requests have retired and others were admitted after
    while frame[0] < 20:
        while pending and pending[0][0] <= frame[0]:
            srv.submit(pending.pop(0)[1])
        srv.admit()
        before = srv.frames
        srv.step_chunk()
        frame[0] += max(srv.frames - before, 1)
    srv.admit()
    assert len(srv.done) >= 2 and len(srv.resident) >= 2
    b = srv.batch
    picks = [0, len(srv.resident) - 1]
    states = {}
    for i in picks:
        states[i] = b.copy_out_scene(i, gsph.FIELD_POSITION)
    assert any(b.pbase[i] > 0 for i in picks)   # a scene away from the batch start
    b.arrange()
    b.density()
    b.force()
    for i in picks:
        r = srv.resident[i]
        _scene_checks(gsph, oracle, b, i, r.params, states[i])
    srv.close()
