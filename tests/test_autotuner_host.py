"""The Python autotuner's host side on CPU: the occupancy signature it caches
tunings under, and the cache itself, driven through a stand-in handle (the
trials themselves are GPU work, covered by test_gpu_tuning.py)."""
import numpy as np


def test_occupancy_signature_bins(gsph):
    # occupied counts 1 | 2 3 | 4 7 | 8 | 600 (>= 512 shares the last bin)
    counts = np.array([0, 1, 2, 3, 4, 7, 8, 600, 0, 0], np.int32)
    sig = gsph.occupancy_signature(counts, 625)
    assert sig[0] == 9                       # floor(log2(625))
    frac = sig[1:]
    assert len(frac) == 10
    assert frac[0] == 0.15 and frac[1] == 0.3 and frac[2] == 0.3
    assert frac[3] == 0.15 and frac[9] == 0.15
    assert abs(sum(frac) - 1.0) < 0.11       # rounded to 0.05 each
    assert gsph.occupancy_signature(np.zeros(5, np.int32), 0) == (0,)


def test_signature_ignores_placement_but_not_occupancy(gsph):
    rng = np.random.default_rng(2)
    counts = rng.integers(0, 12, 5000).astype(np.int32)
    moved = rng.permutation(counts)
    assert gsph.occupancy_signature(counts, 30000) == gsph.occupancy_signature(moved, 30000)
    crowded = counts * 8
    assert gsph.occupancy_signature(counts, 30000) != gsph.occupancy_signature(crowded, 30000)


class _Handle:
    """What Autotuner calls on a handle: arrange, copy_out(cell counts), n,
    autotune and set_tuning."""

    def __init__(self, counts, tuning):
        self.counts = np.asarray(counts, np.int32)
        self.n = int(self.counts.sum())
        self.tuning = tuning
        self.autotuned = 0
        self.installed = None

    def arrange(self):
        pass

    def copy_out(self, field):
        return self.counts

    def autotune(self, frames, candidates):
        self.autotuned += 1
        return self.tuning, 1.25

    def set_tuning(self, t):
        self.installed = t


def test_autotuner_caches_by_signature(gsph):
    tuner = gsph.Autotuner(frames_per_trial=1)
    best = gsph.tuning_default()
    best.warps_per_block = 4
    a = _Handle([8] * 100 + [0] * 50, best)
    t, ms, cached = tuner.tune(a)
    assert not cached and a.autotuned == 1 and t.warps_per_block == 4 and ms == 1.25
    # same occupancy (other cells, same histogram): the cached tuning, no trials
    b = _Handle([0] * 50 + [8] * 100, gsph.tuning_default())
    t, ms, cached = tuner.tune(b)
    assert cached and b.autotuned == 0 and b.installed.warps_per_block == 4
    # another occupancy: a new search
    c = _Handle([40] * 100, gsph.tuning_default())
    t, ms, cached = tuner.tune(c)
    assert not cached and c.autotuned == 1
