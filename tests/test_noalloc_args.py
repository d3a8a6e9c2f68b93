"""Argument checks of the grid-sort entry points, on the CPU.

Every check below runs before the library touches CUDA, so these calls launch
nothing and need no GPU: a grid with a non-positive or oversized dimension, or
with more cells than the 32-bit micro key holds, is refused with a status
code. The no-allocation sort's fixed scratch array must also hold the scratch
layout of its declared maximum input.
"""
import ctypes as C
import re
from pathlib import Path

import pytest

from gpu_helpers import dam_scene

HEADER = Path(__file__).resolve().parent.parent / "include" / "gsph.h"


def header_define(name):
    return int(re.search(rf"#define {name} (\d+)u", HEADER.read_text()).group(1))


def test_noalloc_scratch_holds_the_declared_maximum(gsph):
    lib = gsph.load_library()
    need = lib.gsph_grid_sort_scratch_bytes(header_define("GSPH_NOALLOC_MAX_PARTICLES"),
                                            header_define("GSPH_NOALLOC_MAX_CELLS"))
    assert need <= header_define("GSPH_NOALLOC_SCRATCH_BYTES")


BAD_GRIDS = [
    ((-1, -1, 100), "ERR_INVALID_ARG"),     # two negative dimensions, positive product
    ((0, 10, 10), "ERR_INVALID_ARG"),
    ((10, -3, 10), "ERR_INVALID_ARG"),
    ((65536, 1, 1), "ERR_INVALID_ARG"),     # beyond the 16-bit task cell position
    ((65535, 65535, 65535), "ERR_CAPACITY"),   # overflows a 32-bit product
    ((1024, 256, 256), "ERR_CAPACITY"),     # 2^26 cells: key space exceeded
]


@pytest.mark.parametrize("grid,err", BAD_GRIDS)
def test_grid_sorts_refuse_bad_grids_without_launching(gsph, grid, err):
    lib = gsph.load_library()
    _, p, _ = dam_scene(gsph, n_side=4)
    q = gsph.Params.from_buffer_copy(p)
    for a in range(3):
        q.grid_size[a] = grid[a]
    dummy = C.c_float * 16
    buf = dummy()
    ptr = C.addressof(buf)
    st = lib.gsph_grid_sort_dev_noalloc(C.byref(q), 8, ptr, ptr, ptr, ptr, ptr, ptr,
                                        ptr, ptr, ptr, None)
    assert st == getattr(gsph, err), lib.gsph_last_error()
    assert b"grid" in lib.gsph_last_error()
    st = lib.gsph_grid_sort_dev(C.byref(q), 8, ptr, ptr, ptr, ptr, ptr, ptr, ptr, ptr,
                                ptr, ptr, 1 << 20, None)
    assert st == getattr(gsph, err), lib.gsph_last_error()
