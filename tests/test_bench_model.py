"""bench.py's roofline inputs on CPU: the cell-tile byte model against a
direct count, the per-workload traffic lookup, and the committed traffic
figures against the ncu summaries they come from."""
import re
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_tile_bytes_matches_a_direct_count():
    rng = np.random.default_rng(3)
    gx, gy, gz = 7, 5, 4
    counts = rng.integers(0, 6, size=gx * gy * gz)
    counts[rng.random(counts.size) < 0.3] = 0
    n = int(counts.sum())
    s = 0
    for z in range(gz):
        for y in range(gy):
            for x in range(gx):
                c = x + gx * (y + gy * z)
                if counts[c] == 0:
                    continue
                for dz in (-1, 0, 1):
                    for dy in (-1, 0, 1):
                        for dx in (-1, 0, 1):
                            X, Y, Z = x + dx, y + dy, z + dz
                            if 0 <= X < gx and 0 <= Y < gy and 0 <= Z < gz:
                                s += int(counts[X + gx * (Y + gy * Z)])
    b_den, b_for = bench.tile_bytes(counts, (gx, gy, gz), n)
    assert b_den == 16 * s + 24 * n
    assert b_for == 32 * s + 44 * n


def test_traffic_lookup_is_per_workload():
    assert bench.ncu_traffic("k_force_tra", "dam_break_3_94m") > 0
    assert 0 < bench.ncu_traffic("k_density_tra", "dam_break_3_94m", "fma_pipe") < 1
    # no capture of another workload: no figure, rather than a borrowed one
    assert bench.ncu_traffic("k_force_tra", "stress") is None
    assert bench.ncu_traffic("k_no_such_kernel", "dam_break_3_94m") is None


def test_committed_traffic_matches_the_profiles():
    """Every `kernel@workload = bytes` line equals DRAM read + write of the
    full capture summarised in profiles/<kernel>_<scene>.md."""
    lines = (ROOT / "profiles" / "traffic_per_launch.txt").read_text().splitlines()
    entries = [re.match(r"(k_\w+)@(\w+)\s*=\s*([0-9]+)$", l.strip()) for l in lines]
    entries = [m for m in entries if m]
    assert len(entries) >= 4
    for m in entries:
        kernel, workload, value = m.group(1), m.group(2), int(m.group(3))
        md = (ROOT / "profiles" / f"{kernel}_{workload}.md").read_text()
        rd = float(re.search(r"dram__bytes_read\.sum`\) \| ([0-9.]+) \| Mbyte", md).group(1))
        wr = float(re.search(r"dram__bytes_write\.sum`\) \| ([0-9.]+) \| Mbyte", md).group(1))
        assert abs((rd + wr) * 1e6 - value) < 1e3, (kernel, workload)
