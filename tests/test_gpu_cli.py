"""The `gsph` command: the reference's headless benchmark flags and print
block (src/main.cpp:42-85, sph_hybrid_system.cpp:397-429), with the state
checksum of the same frames stepped through the library."""
import re
import subprocess

import numpy as np
import pytest

from gpu_helpers import dam_scene_text

pytestmark = pytest.mark.gpu


def _run(gsph, args):
    exe = gsph.PKG_DIR / "lib" / "gsph"
    r = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=300)
    return r.returncode, r.stdout, r.stderr


def test_benchmark_block_and_checksum(gsph, cuda_device, tmp_path):
    scene = tmp_path / "scene.json"
    scene.write_text(dam_scene_text(n_side=18, seed=4))
    rc, out, err = _run(gsph, ["--benchmark", "9", "--scene", str(scene)])
    assert rc == 0, err
    assert "CUDA initialized." in out
    m = re.search(r"Headless benchmark \((\d+) measured \+ (\d+) warm-up frames\)", out)
    assert m and int(m.group(1)) + int(m.group(2)) == 9
    for line in ("Total wall time:", "Average frame time:", "FPS:", "Hybrid split:",
                 "judgeTask isSame SMS pairs:", "Per-stage averages", "arrange/grid :",
                 "density      :", "force        :"):
        assert line in out, line
    cs = re.search(r"State checksum: (\S+), (\S+), (\S+), (\S+), (\S+)", out)
    got = np.array([float(x) for x in cs.groups()])
    n = int(re.search(r"Number of particles: (\d+)", out).group(1))
    split = re.search(r"Hybrid split: (\d+) TRA particles, (\d+) SMS tasks", out)
    assert int(split.group(1)) == n and int(split.group(2)) == 0
    with gsph.HybridSystem(scene) as h:
        assert h.n == n
        h.step(9)
        want = np.array(h.checksum())
    assert np.array_equal(got, want)
    # graph launches (10 frames per graph) give the same state
    rc, out2, err = _run(gsph, ["--benchmark", "25", "--scene", str(scene), "--graph"])
    assert rc == 0, err
    with gsph.HybridSystem(scene) as h:
        h.step(25)
        want25 = np.array(h.checksum())
    cs2 = re.search(r"State checksum: (\S+), (\S+), (\S+), (\S+), (\S+)", out2)
    assert np.array_equal(np.array([float(x) for x in cs2.groups()]), want25)


def test_bad_arguments_fail_cleanly(gsph, cuda_device, tmp_path):
    rc, out, err = _run(gsph, ["--benchmark", "0"])
    assert rc != 0 and "positive" in err
    rc, out, err = _run(gsph, ["--benchmark", "3", "--scene", str(tmp_path / "missing.json")])
    assert rc != 0 and err.strip()


def test_cli_artificial_viscosity_and_autotune(gsph, cuda_device, tmp_path):
    scene = tmp_path / "scene.json"
    scene.write_text(dam_scene_text(n_side=12, seed=2))
    rc, out, err = _run(gsph, ["--benchmark", "6", "--scene", str(scene),
                               "--artificial-viscosity", "0.02", "20", "--autotune", "--graph"])
    assert rc == 0, err
    assert "Artificial viscosity: alpha 0.02, c0 20" in out
    assert re.search(r"Autotuned: thresholds \d+/\d+/\d+, CTAs per SM \d+/\d+/\d+/\d+, "
                     r"[48] warps per block", out)
    assert "FPS:" in out
    rc, out, err = _run(gsph, ["--benchmark", "3", "--scene", str(scene),
                               "--artificial-viscosity", "0", "20"])
    assert rc != 0 and "alpha and c0" in err
