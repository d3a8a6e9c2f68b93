"""The no-allocation grid sort (gsph_grid_sort_dev_noalloc).

Callers that cannot allocate device memory at the call site — hosts held to a
fixed device-memory budget by their own pool allocator, and real-time loops
that cannot afford cudaMalloc's implicit synchronisation — use this entry
point: it takes only inputs and outputs and keeps its scratch in a fixed
device array inside the library. This file is collected last so that a run
stopping at its first failure has already run every other test.

The check: two calls in a row on different inputs, each compared with the
allocating entry point (gsph_grid_sort_dev with caller scratch) on the same
input. Integer outputs and the copied particle records must be identical (the
tolerance used for the grid stage everywhere: bit-exact).
"""
import ctypes as C

import numpy as np
import pytest

from gpu_helpers import dam_scene, shuffled

pytestmark = pytest.mark.gpu


def _outputs(torch, n, numc, dev):
    f4 = lambda: torch.empty((n, 4), dtype=torch.float32, device=dev)
    return {
        "pos": f4(), "vel": f4(), "ev": f4(),
        "key": torch.empty(n, dtype=torch.int32, device=dev),
        "perm": torch.empty(n, dtype=torch.int32, device=dev),
        "cs": torch.empty(numc + 1, dtype=torch.int32, device=dev),
    }


def _host(o):
    return {k: v.cpu().numpy() for k, v in o.items()}


def test_noalloc_grid_sort_matches_allocating_sort(gsph, cuda_device):
    import torch

    lib = gsph.load_library()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    s, p, base = dam_scene(gsph, n_side=28, box=(0.8, 0.5, 0.5))
    n, numc = len(base), p.numc
    assert n <= gsph_max(lib, "particles") and numc <= gsph_max(lib, "cells")
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(3)

    for call in range(2):
        pos = shuffled(base, seed=100 + call)
        vel = rng.normal(0, 1, pos.shape).astype(np.float32)
        ev = rng.normal(0, 1, pos.shape).astype(np.float32)
        pin, vin, ein = (torch.from_numpy(a).to(dev) for a in (pos, vel, ev))

        # allocating entry point, caller scratch
        ref = _outputs(torch, n, numc, dev)
        nbytes = lib.gsph_grid_sort_scratch_bytes(n, numc)
        scratch = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
        base_ptr = (scratch.data_ptr() + 255) // 256 * 256
        st = lib.gsph_grid_sort_dev(C.byref(p), n, pin.data_ptr(), vin.data_ptr(),
                                    ein.data_ptr(), ref["pos"].data_ptr(),
                                    ref["vel"].data_ptr(), ref["ev"].data_ptr(),
                                    ref["key"].data_ptr(), ref["perm"].data_ptr(),
                                    ref["cs"].data_ptr(), base_ptr, nbytes, stream)
        assert st == 0, lib.gsph_last_error()

        # no-allocation entry point
        out = _outputs(torch, n, numc, dev)
        st = lib.gsph_grid_sort_dev_noalloc(C.byref(p), n, pin.data_ptr(), vin.data_ptr(),
                                            ein.data_ptr(), out["pos"].data_ptr(),
                                            out["vel"].data_ptr(), out["ev"].data_ptr(),
                                            out["key"].data_ptr(), out["perm"].data_ptr(),
                                            out["cs"].data_ptr(), stream)
        assert st == 0, lib.gsph_last_error()
        torch.cuda.synchronize()
        a, b = _host(ref), _host(out)
        for k in a:
            assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), (call, k)
        # and the sort is a real one: keys ascending, records follow the permutation
        assert np.all(np.diff(b["key"].view(np.uint32).astype(np.int64)) >= 0)
        assert np.array_equal(b["pos"], pos[b["perm"]])


def test_noalloc_at_the_declared_maximum(gsph, cuda_device):
    """The 262,144-particle dam break over its 128 x 64 x 64 = 524,288-cell grid
    is exactly the declared maximum: the scratch layout then fills the array."""
    import torch

    lib = gsph.load_library()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    s = gsph.load_scene(gsph.scene_path("dam_break_262k.json"))
    p = gsph.params_init(s)
    base = gsph.lattice(s, p)
    n, numc = len(base), p.numc
    assert n == gsph_max(lib, "particles") and numc == gsph_max(lib, "cells")
    stream = torch.cuda.current_stream().cuda_stream
    pos = shuffled(base, seed=7)
    vel = np.zeros_like(pos)
    pin, vin = (torch.from_numpy(a).to(dev) for a in (pos, vel))
    ref = _outputs(torch, n, numc, dev)
    nbytes = lib.gsph_grid_sort_scratch_bytes(n, numc)
    scratch = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
    base_ptr = (scratch.data_ptr() + 255) // 256 * 256
    st = lib.gsph_grid_sort_dev(C.byref(p), n, pin.data_ptr(), vin.data_ptr(),
                                vin.data_ptr(), ref["pos"].data_ptr(), ref["vel"].data_ptr(),
                                ref["ev"].data_ptr(), ref["key"].data_ptr(),
                                ref["perm"].data_ptr(), ref["cs"].data_ptr(), base_ptr,
                                nbytes, stream)
    assert st == 0, lib.gsph_last_error()
    for call in range(2):
        out = _outputs(torch, n, numc, dev)
        st = lib.gsph_grid_sort_dev_noalloc(C.byref(p), n, pin.data_ptr(), vin.data_ptr(),
                                            vin.data_ptr(), out["pos"].data_ptr(),
                                            out["vel"].data_ptr(), out["ev"].data_ptr(),
                                            out["key"].data_ptr(), out["perm"].data_ptr(),
                                            out["cs"].data_ptr(), stream)
        assert st == 0, lib.gsph_last_error()
        torch.cuda.synchronize()
        a, b = _host(ref), _host(out)
        for k in a:
            assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), (call, k)


def test_noalloc_rejects_sizes_beyond_its_scratch(gsph, cuda_device):
    import torch

    lib = gsph.load_library()
    s, p, pos = dam_scene(gsph, n_side=8)
    dummy = torch.empty(16, dtype=torch.float32, device="cuda")
    ptr = dummy.data_ptr()
    too_many = gsph_max(lib, "particles") + 1
    st = lib.gsph_grid_sort_dev_noalloc(C.byref(p), too_many, ptr, ptr, ptr, ptr, ptr, ptr,
                                        ptr, ptr, ptr, None)
    assert st == gsph.ERR_CAPACITY
    assert b"exceed" in lib.gsph_last_error()
    big = gsph.Params.from_buffer_copy(p)
    big.grid_size[0] = 4096          # 4096 * 25 * 25 cells > maximum
    big.grid_size[1] = big.grid_size[2] = 25
    st = lib.gsph_grid_sort_dev_noalloc(C.byref(big), 10, ptr, ptr, ptr, ptr, ptr, ptr,
                                        ptr, ptr, ptr, None)
    assert st == gsph.ERR_CAPACITY


def gsph_max(lib, what):
    """The limits declared in include/gsph.h."""
    import re
    from pathlib import Path
    text = (Path(__file__).resolve().parent.parent / "include" / "gsph.h").read_text()
    name = {"particles": "GSPH_NOALLOC_MAX_PARTICLES", "cells": "GSPH_NOALLOC_MAX_CELLS"}[what]
    return int(re.search(rf"#define {name} (\d+)u", text).group(1))
