"""The CPU oracle checked against independent restatements and known answers
(no GPU). The oracle itself is pinned to reference outputs by
tests/test_golden.py."""
import math

import numpy as np
import pytest


def small_scene(gsph, n_side=12, jitter=0.05, box=(0.6, 0.4, 0.4), seed=3,
                begin=0.055, kernel=0.02):
    end = begin + n_side * kernel * 0.5 - kernel * 0.25
    text = f'''{{"fluid_block": [{{"begin_x": {begin}, "begin_y": {begin}, "begin_z": {begin},
        "end_x": {end}, "end_y": {end}, "end_z": {end}}}],
        "mass": 0.001, "interval": 0.5, "kernel": {kernel}, "gas_constant": 57142.857,
        "viscosity": 0.8, "time_step": 0.0001, "gravity_y": -9.81,
        "jitter": {jitter}, "seed": {seed}, "xx": {box[0]}, "yy": {box[1]}, "zz": {box[2]}}}'''
    s = gsph.parse_scene(text)
    p = gsph.params_init(s)
    return s, p, gsph.lattice(s, p)


def numpy_keys(pos, p):
    """Third restatement of sph_utils.cuh:44-99 with numpy float32 math."""
    rat = np.float32(4.0) * np.float32(p.inv_cell_size)
    m = np.floor(pos[:, :3].astype(np.float32) * rat).astype(np.int64)
    gx, gy, gz = (int(g) for g in p.grid_size)
    c = (m[:, 0] >> 2) + gx * ((m[:, 1] >> 2) + gy * (m[:, 2] >> 2))
    sub = (m[:, 1] & 3) + (((m[:, 2] & 3) + ((m[:, 0] & 3) << 2)) << 2)
    return ((c << 6) | sub).astype(np.uint32)


def test_keys_match_numpy(gsph, oracle):
    s, p, pos = small_scene(gsph)
    assert np.array_equal(oracle.keys(pos, p), numpy_keys(pos, p))


def test_key_layout_known_answer(gsph, oracle):
    s, p, _ = small_scene(gsph)
    h = float(p.kernel)
    # micro cell (mx, my, mz) = (5, 2, 7): coarse (1, 0, 1), local (1, 2, 3)
    pos = np.array([[5.5 * h / 4, 2.5 * h / 4, 7.5 * h / 4, 0]], np.float32)
    gx, gy = p.grid_size[0], p.grid_size[1]
    c = 1 + gx * (0 + gy * 1)
    assert oracle.keys(pos, p)[0] == (c << 6) | (1 << 4) | (3 << 2) | 2


def test_sort_is_stable_counting_sort(gsph, oracle):
    s, p, pos = small_scene(gsph)
    rng = np.random.default_rng(0)
    pos = pos[rng.permutation(len(pos))]
    ks, perm, cs, bad = oracle.sort(pos, p)
    assert not bad
    k = oracle.keys(pos, p)
    assert np.array_equal(np.sort(perm), np.arange(len(pos)))
    assert np.array_equal(ks, k[perm])
    order = np.lexsort((np.arange(len(pos)), k))
    assert np.array_equal(perm, order)
    counts = np.bincount((k >> 6).astype(np.int64), minlength=oracle.numc(p))
    assert np.array_equal(np.diff(cs), counts)
    ms = oracle.micro_start(ks, p)
    assert ms[-1] == len(pos)
    # micro cell ranges hold exactly their keys
    for key in np.unique(ks)[:50]:
        a, b = ms[key], ms[key + 1]
        assert np.all(ks[a:b] == key)


def synthetic_starts(counts):
    cs = np.zeros(len(counts) + 1, np.int32)
    np.cumsum(counts, out=cs[1:])
    return cs


def test_block_req_thresholds(gsph, oracle):
    # gpu_model.cu:172-180 on a 5x5x5 grid, probing the centre cell
    s, p, _ = small_scene(gsph)
    p.grid_size[0] = p.grid_size[1] = p.grid_size[2] = 5
    centre = 2 + 5 * (2 + 5 * 2)
    nbrs = [centre - 1, centre + 1, centre - 5, centre + 5, centre - 25, centre + 25]

    def req(self_n, nbr_n):
        c = np.zeros(125, np.int32)
        c[centre] = self_n
        for q in nbrs:
            c[q] = nbr_n
        return oracle.block_req(synthetic_starts(c), p)[centre]

    assert req(14, 13) == 0            # total 92 < 96 and self < 15
    assert req(14, 14) == 1            # total 98: (14+31)>>5
    assert req(15, 0) == 1             # total < 60: (15+27)>>5
    assert req(36, 3) == 1             # total 54 < 60: 36 particles, 1 task
    assert req(37, 3) == 2
    assert req(33, 5) == 2             # total 63: (33+31)>>5
    assert req(0, 50) == 0
    assert req(64, 10) == 2
    assert req(65, 10) == 3
    # corner cell: missing neighbours are skipped, not wrapped
    c = np.zeros(125, np.int32)
    c[0] = 20
    c[1] = 40
    c[124] = 1000
    r = oracle.block_req(synthetic_starts(c), p)
    assert r[0] == (20 + 31) >> 5 and r[124] == (1000 + 31) >> 5


def test_split_and_tasks(gsph, oracle):
    s, p, _ = small_scene(gsph)
    p.grid_size[0], p.grid_size[1], p.grid_size[2] = 4, 1, 1
    counts = np.array([70, 5, 35, 0], np.int32)
    cs = synthetic_starts(counts)
    req = np.array([3, 0, 1, 0], np.int32)
    compact, middle = oracle.split(cs, req, p)
    # TRA: cell 1 (5 particles) + cell 2 tail (3); SMS: cell 0 (70), cell 2 (32)
    assert middle == 8
    assert list(compact[:8]) == [70, 71, 72, 73, 74, 107, 108, 109]
    assert list(compact[8:78]) == list(range(70))
    assert list(compact[78:]) == list(range(75, 107))
    # keys: cell 0 particles sorted over micro x 0..3; cell 2 all in micro x 1
    ks = np.zeros(cs[-1], np.uint32)
    ks[:70] = (0 << 6) | (np.repeat([0, 1, 2, 3], [20, 20, 20, 10]) << 4) | 5
    ks[70:75] = (1 << 6)
    ks[75:110] = (2 << 6) | (1 << 4) | (2 << 2) | np.arange(35) % 4
    ks[75:110].sort()
    t = oracle.tasks(ks, cs, req, p, gsph.BLOCK_TASK_DTYPE)
    assert len(t) == 4                                  # 4 tasks, even
    assert list(t["cellid"]) == [0, 0, 0, 2]
    assert list(t["p_offset"]) == [0, 32, 64, 0]
    assert (t["xxi"][0], t["xxx"][0]) == (0, 1)        # spans x: full y/z
    assert (t["zzi"][0], t["zzz"][0], t["yyi"][0], t["yyy"][0]) == (0, 3, 0, 3)
    assert (t["xxi"][3], t["xxx"][3], t["zzi"][3], t["zzz"][3]) == (1, 1, 2, 2)
    assert (t["yyi"][3], t["yyy"][3]) == (0, 3)
    # judgeTask: (0,1) same cell, (2,3) different cells
    assert list(t["is_same"]) == [1, 1, 0, 0]
    pb = int(t["paired_bounds"][0])
    assert (pb & 3, (pb >> 2) & 3) == (t["xxi"][0], t["xxx"][1])
    # odd count: a pad descriptor of the same cell, p_offset + 32
    t3 = oracle.tasks(ks, cs, np.array([3, 0, 0, 0], np.int32), p, gsph.BLOCK_TASK_DTYPE)
    assert len(t3) == 4 and t3["p_offset"][3] == 96 and t3["cellid"][3] == 0
    assert t3["is_same"][2] == 1 and t3["is_same"][3] == 1


def brute_density(pos, p):
    x = pos[:, :3].astype(np.float64)
    d2 = ((x[:, None, :] - x[None, :, :]) ** 2).sum(-1)
    h2 = float(p.kernel) ** 2
    w = np.where((d2 <= h2) & (d2 >= 1e-12), (h2 - d2) ** 3, 0.0)
    return w.sum(1) * float(p.density_scale) + float(p.self_density)


def test_density_matches_brute_force(gsph, oracle):
    s, p, pos = small_scene(gsph, n_side=10)
    ks, perm, cs, _ = oracle.sort(pos, p)
    sp = pos[perm]
    rho, pr = oracle.density(sp, ks, cs, p)
    ref = brute_density(sp, p)
    np.testing.assert_allclose(rho, ref, rtol=1e-12)
    np.testing.assert_allclose(
        pr, ((ref / float(p.rest_density)) ** 7 - 1) * float(p.gas_constant), rtol=1e-9)


def test_density_of_interior_lattice(gsph, oracle):
    # cubic lattice, spacing h/2: sum over the 32 neighbours within h
    s, p, pos = small_scene(gsph, n_side=14, jitter=0.0)
    ks, perm, cs, _ = oracle.sort(pos, p)
    rho, _ = oracle.density(pos[perm], ks, cs, p)
    dx, h = 0.01, float(p.kernel)
    r = np.arange(-2, 3) * dx
    d2 = (r[:, None, None] ** 2 + r[None, :, None] ** 2 + r[None, None, :] ** 2).ravel()
    w = sum((h * h - d) ** 3 for d in d2 if 1e-12 <= d <= h * h)
    expect = w * float(p.density_scale) + float(p.self_density)
    assert abs(np.max(rho) - expect) / expect < 1e-4
    assert 1000.0 < expect < 1020.0


def test_force_momentum_balance(gsph, oracle):
    # pressure and viscosity pair terms are antisymmetric once divided by
    # rho_i: sum_i F_i / rho_i = 0 (surface tension switched off)
    s, p, pos = small_scene(gsph, n_side=10)
    p.surface_coe = 0.0
    ks, perm, cs, _ = oracle.sort(pos, p)
    sp = pos[perm].copy()
    rho, pr = oracle.density(sp, ks, cs, p)
    sp[:, 3] = (1.0 / rho).astype(np.float32)
    rng = np.random.default_rng(1)
    ev = np.zeros_like(sp)
    ev[:, :3] = rng.normal(0, 0.1, (len(sp), 3))
    ev[:, 3] = pr.astype(np.float32)
    acc = oracle.force(sp, ev, ks, cs, p)
    net = (acc * sp[:, 3:4].astype(np.float64)).sum(0)
    scale = np.abs(acc * sp[:, 3:4]).sum(0)
    assert np.all(np.abs(net) <= 1e-9 * scale + 1e-12)


def test_integrate_walls_and_clamps(gsph, oracle):
    s, p, _ = small_scene(gsph)
    pos = np.array([[0.03, 0.2, 0.2, 1e-3],      # inside the penalty zone at x-min
                    [0.3, 0.2, 0.2, 1e-3],       # free fall
                    [0.3, 0.2, 0.2, 1e-3]], np.float64)
    vel = np.zeros((3, 4))
    vel[2, 0] = 100.0                            # speed clamp (|v| <= 6)
    ev = np.zeros((3, 4))
    acc = np.zeros((3, 3))
    P, V, E = oracle.integrate(pos, vel, ev, acc, p)
    assert V[0, 0] > 0                           # pushed away from the wall
    assert math.isclose(V[1, 1], -9.81 * 1e-4, rel_tol=1e-6)
    assert math.isclose(np.linalg.norm(V[2, :3]), 6.0, rel_tol=1e-9)
    assert np.allclose(E[:, :3], V[:, :3] / 2)
    assert np.all(P[:, 3] == pos[:, 3])


def test_step_is_deterministic_and_conserves_count(gsph, oracle):
    s, p, pos = small_scene(gsph, n_side=8)
    vel = np.zeros_like(pos)
    ev = np.zeros_like(pos)
    a = oracle.step(pos, vel, ev, p, 3)
    b = oracle.step(pos, vel, ev, p, 3)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert len(a[0]) == len(pos)
    assert np.all(np.isfinite(a[0]))
    assert oracle.num_threads() >= 1


def _force_inputs(oracle, p, pos, seed=1, v_scale=0.1):
    ks, perm, cs, _ = oracle.sort(pos, p)
    sp = pos[perm].copy()
    rho, pr = oracle.density(sp, ks, cs, p)
    sp[:, 3] = (1.0 / rho).astype(np.float32)
    rng = np.random.default_rng(seed)
    ev = np.zeros_like(sp)
    ev[:, :3] = rng.normal(0, v_scale, (len(sp), 3))
    ev[:, 3] = pr.astype(np.float32)
    return sp, ev, ks, cs


def brute_viscosity(sp, ev, p, alpha=None, c0=None):
    """Viscosity part of the force, all pairs in numpy FP64: the reference's
    Laplacian form m mu visco sum V_j (v_j - v_i)(h - r), or Monaghan's
    artificial viscosity -m rho_i sum Pi_ij grad W_spiky (Monaghan 1992)."""
    x = sp[:, :3].astype(np.float64)
    v = ev[:, :3].astype(np.float64)
    V = sp[:, 3].astype(np.float64)
    r = x[:, None, :] - x[None, :, :]
    d2 = (r ** 2).sum(-1)
    h = float(p.kernel)
    inside = (d2 <= h * h) & (d2 >= 1e-12)
    d = np.sqrt(np.where(inside, d2, 1.0))
    k = np.where(inside, h - d, 0.0)
    m = float(p.mass)
    if alpha is None:
        w = V[None, :] * k
        return m * float(p.viscosity_visco_value) * (w[:, :, None] * (v[None, :, :] - v[:, None, :])).sum(1)
    vr = ((v[:, None, :] - v[None, :, :]) * r).sum(-1)
    mu = h * vr / (d2 + float(np.float32(0.01) * np.float32(p.kernel_2)))
    rho_mean = 0.5 * (1.0 / V[:, None] + 1.0 / V[None, :])
    coef = float(np.float32(alpha) * np.float32(c0))
    pij = np.where(inside & (vr < 0), -coef * mu / rho_mean, 0.0)
    grad = float(p.spiky_value) * (k * k / d)[:, :, None] * r       # spiky gradient
    return -m / V[:, None] * (pij[:, :, None] * grad).sum(1)


def test_artificial_viscosity_matches_brute_force(gsph, oracle):
    """The oracle's two viscosity models differ exactly by the difference of
    the two brute-force viscosity terms (everything else is shared)."""
    s, p, pos = small_scene(gsph, n_side=9)
    sp, ev, ks, cs = _force_inputs(oracle, p, pos, v_scale=0.3)
    lap = oracle.force(sp, ev, ks, cs, p)
    art = oracle.force(sp, ev, ks, cs, p, artificial=(0.02, 20.0))
    expect = brute_viscosity(sp, ev, p, 0.02, 20.0) - brute_viscosity(sp, ev, p)
    scale = np.abs(expect).max()
    assert scale > 0
    np.testing.assert_allclose(art - lap, expect, rtol=0, atol=1e-9 * scale)
    # approaching pairs only: with all particles receding from the centre the
    # artificial term vanishes
    c = sp[:, :3].astype(np.float64).mean(0)
    ev2 = ev.copy()
    ev2[:, :3] = (sp[:, :3] - c).astype(np.float32)
    assert np.abs(brute_viscosity(sp, ev2, p, 0.02, 20.0)).max() == 0.0


def test_artificial_viscosity_momentum_balance(gsph, oracle):
    s, p, pos = small_scene(gsph, n_side=10)
    p.surface_coe = 0.0
    sp, ev, ks, cs = _force_inputs(oracle, p, pos, v_scale=0.5)
    acc = oracle.force(sp, ev, ks, cs, p, artificial=(0.5, 20.0))
    net = (acc * sp[:, 3:4].astype(np.float64)).sum(0)
    scale = np.abs(acc * sp[:, 3:4]).sum(0)
    assert np.all(np.abs(net) <= 1e-9 * scale + 1e-12)
