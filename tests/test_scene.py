"""Scene loader, parameters and lattice (row A1) — host code, no GPU.

The library's host side must agree bit for bit with the oracle's restatement
of readSceneFromJsonFile / defaultInitializeSPHSysPara / initializeScene
(src/simulation/sph_hybrid_system.cpp:69-202, 432-473 of the reference).
"""
import ctypes as C
import math

import numpy as np
import pytest


SCENES = ["scene_default.json", "dam_break_262k.json", "dam_break_3_94m.json"]


def _fields(p):
    out = {}
    for name, typ in type(p)._fields_:
        v = getattr(p, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


@pytest.mark.parametrize("name", SCENES)
def test_params_match_oracle(gsph, oracle, name):
    scene = gsph.load_scene(gsph.scene_path(name))
    mine = gsph.params_init(scene)
    ref = oracle.params_init(scene, gsph.Params)
    a, b = _fields(mine), _fields(ref)
    for k in a:
        va, vb = np.asarray(a[k]), np.asarray(b[k])
        assert np.array_equal(va.view(np.uint32) if va.dtype == np.float32 else va,
                              vb.view(np.uint32) if vb.dtype == np.float32 else vb) or \
            np.array_equal(va, vb), k


def test_default_scene_constants(gsph):
    # Reference hard-coded physics (sph_hybrid_system.cpp:136-193).
    s = gsph.load_scene(gsph.scene_path("scene_default.json"))
    p = gsph.params_init(s)
    assert p.kernel == np.float32(0.03)
    assert list(p.grid_size) == [54, 54, 54]
    assert p.gas_constant == 1.0 and p.rest_density == 1000.0
    assert p.time_step == np.float32(0.003) and p.viscosity == np.float32(6.5)
    assert p.gravity[1] == np.float32(-9.8)
    k = float(np.float32(0.03))
    assert p.poly6_value == np.float32(315.0 / (64.0 * math.pi * k ** 9))
    assert p.half_spiky_value == np.float32(p.spiky_value * np.float32(0.5))
    assert p.bound_min[0] == p.kernel
    assert p.bound_max[0] == np.float32(np.float32(1.6) - np.float32(0.03))


@pytest.mark.parametrize("name,count", [("scene_default.json", 3944312),
                                        ("dam_break_262k.json", 64 ** 3),
                                        ("dam_break_3_94m.json", 158 ** 3)])
def test_lattice_counts(gsph, name, count):
    s = gsph.load_scene(gsph.scene_path(name))
    p = gsph.params_init(s)
    n = C.c_uint32()
    assert gsph.load_library().gsph_lattice_count(C.byref(s), C.byref(p), C.byref(n)) == 0
    assert n.value == count


def test_lattice_matches_oracle_without_jitter(gsph, oracle):
    s = gsph.load_scene(gsph.scene_path("scene_default.json"))
    p = gsph.params_init(s)
    mine = gsph.lattice(s, p)
    ref = oracle.lattice(s, p)
    assert mine.shape == ref.shape
    assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32))
    # order x outer, y, z inner
    assert mine[1, 2] > mine[0, 2] and mine[1, 0] == mine[0, 0]


def test_lattice_jitter_bounded_and_seeded(gsph, oracle):
    s = gsph.load_scene(gsph.scene_path("dam_break_262k.json"))
    p = gsph.params_init(s)
    jit = gsph.lattice(s, p)
    s.jitter = 0.0
    base = oracle.lattice(s, p)
    step = float(np.float32(p.kernel) * np.float32(s.interval))
    d = jit[:, :3].astype(np.float64) - base[:, :3]
    assert np.abs(d).max() <= 0.05 * step + 1e-7   # + float rounding of x
    assert np.abs(d).max() > 0.04 * step          # jitter is actually applied
    assert abs(d.mean()) < 1e-3 * step            # centred
    s.jitter = 0.05
    again = gsph.lattice(s, p)
    assert np.array_equal(again, jit)             # seeded, reproducible
    s.seed = 7
    assert not np.array_equal(gsph.lattice(s, p), jit)


def test_json_parser_edge_cases(gsph):
    s = gsph.parse_scene('{"xx": 1, "yy": 2, "zz": 3}')
    assert list(s.world) == [1, 2, 3]
    assert s.n_blocks == 0
    assert s.interval == np.float32(0.5) and s.mass == np.float32(0.02)   # defaults
    assert s.recomm_nump == 65536
    assert math.isnan(s.kernel)
    s = gsph.parse_scene('// comment\n{"fluid_block": [{"begin_x": 0.5, "end_x": 1}],'
                         ' /* c */ "mass": true, "extra": {"a": [1, 2, {"b": null}]}}')
    assert s.n_blocks == 1
    assert s.block_begin[0][0] == 0.5 and s.block_end[0][0] == 1.0
    assert s.block_begin[0][1] == 0.0        # missing member reads as 0 (jsoncpp)
    assert s.mass == 1.0                     # bool -> 1 (jsoncpp asFloat)
    for bad in ['{"xx": }', '{"xx": 1', '[1, 2]', '{"fluid_block": 3}', '', '{"xx": "a"}']:
        with pytest.raises(gsph.GsphError) as ei:
            gsph.parse_scene(bad)
        assert ei.value.status == gsph.ERR_PARSE
    with pytest.raises(gsph.GsphError) as ei:
        gsph.load_scene("/nonexistent/scene.json")
    assert ei.value.status == gsph.ERR_IO


def test_params_rejects_bad_grid(gsph):
    s = gsph.parse_scene('{"xx": 0, "yy": 1, "zz": 1}')
    with pytest.raises(gsph.GsphError) as ei:
        gsph.params_init(s)
    assert ei.value.status == gsph.ERR_INVALID_ARG
    s = gsph.parse_scene('{"xx": 1000, "yy": 1000, "zz": 1000, "kernel": 0.02}')
    with pytest.raises(gsph.GsphError) as ei:
        gsph.params_init(s)
    assert ei.value.status in (gsph.ERR_INVALID_ARG, gsph.ERR_CAPACITY)


@pytest.mark.parametrize("name", SCENES)
def test_oracle_json_reader_matches_library(gsph, oracle, name):
    """The oracle's own scene reader (used where the library must not be
    loaded, e.g. the benchmark's CPU reference arm) gives the same struct."""
    mine = gsph.load_scene(gsph.scene_path(name))
    ref = oracle.scene_from_json(gsph.scene_path(name).read_text(), gsph.Scene)
    assert C.string_at(C.addressof(mine), C.sizeof(mine)) == \
        C.string_at(C.addressof(ref), C.sizeof(ref))
