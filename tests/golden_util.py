"""Loading and canonicalising the reference fixtures in tests/golden/.

The reference orders particles inside a micro cell by atomic slots, which vary
from run to run (src/grid/sph_arrangement.cu:1339). Fixtures are therefore
compared through source identities: every sorted row is mapped back to its
input index by its exact position bits (the fixture scenes have distinct
positions), and within a micro cell the order is made canonical by source
index — the order the oracle and the GB300 library produce.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
SCENES = ["sparse_dam", "dense_default", "mixed", "dam_32k"]


def load(name: str, params_cls):
    d = dict(np.load(GOLDEN / f"{name}.npz"))
    p = params_cls.from_buffer_copy(d["params"].tobytes())
    return d, p


def source_ids(sorted_pos: np.ndarray, in_pos: np.ndarray) -> np.ndarray:
    """Input index of every sorted row, matched by exact position bits."""
    key_in = np.ascontiguousarray(in_pos[:, :3]).view(np.dtype((np.void, 12))).ravel()
    key_s = np.ascontiguousarray(sorted_pos[:, :3]).view(np.dtype((np.void, 12))).ravel()
    order = np.argsort(key_in)
    pos = np.searchsorted(key_in[order], key_s)
    ids = order[np.clip(pos, 0, len(order) - 1)]
    if not np.array_equal(key_in[ids], key_s):
        raise AssertionError("sorted rows do not map one to one onto the input")
    if len(np.unique(ids)) != len(ids):
        raise AssertionError("duplicate positions in fixture input")
    return ids


def canonical_perm(keys: np.ndarray, ids: np.ndarray) -> np.ndarray:
    """Sorted order by (micro key, source index): the canonical permutation."""
    return ids[np.lexsort((ids, keys.astype(np.uint32)))]


def dense_micro(d) -> np.ndarray:
    n_cells = len(d["cell_offset"]) * 64
    out = np.zeros(n_cells + 1, np.int64)
    counts = np.zeros(n_cells, np.int64)
    counts[d["micro_index"]] = d["micro_count"]
    np.cumsum(counts, out=out[1:])
    return out


def split_parts(index: np.ndarray, middle: int, n: int):
    m = n if middle < 0 or middle > n else middle
    return index[:m], index[m:]


def canonical_bucket_ids(part_ids: np.ndarray, cell_of_id: np.ndarray):
    """(cell, id) ordering of one compact-index part, plus whether the part is
    ordered by cell as the reference's bucket scan makes it."""
    cells = cell_of_id[part_ids]
    ordered = bool(np.all(np.diff(cells) >= 0)) if len(cells) else True
    return part_ids[np.lexsort((part_ids, cells))], ordered
