"""Snapshot file format, host side (no GPU): the header reader accepts a file
written to the documented layout and rejects foreign, truncated or
inconsistent files with a status code."""
import ctypes as C
import struct

import numpy as np
import pytest

from gpu_helpers import dam_scene


def _fnv_words(payload: bytes) -> int:
    if len(payload) % 8:
        payload += b"\0" * (8 - len(payload) % 8)
    h = 0xCBF29CE484222325
    for (w,) in struct.iter_unpack("<Q", payload):
        h = ((h ^ w) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def write_snapshot(path, params_list, states, frames=7, version=1):
    counts = [len(s[0]) for s in states]
    pbytes = b"".join(bytes(p) for p in params_list)
    cbytes = np.asarray(counts, np.uint32).tobytes()
    arr = [np.concatenate([s[i] for s in states]).astype(np.float32).tobytes()
           for i in range(3)]
    payload = pbytes + cbytes + b"".join(arr)
    n = sum(counts)
    hdr = struct.pack("<8sIIIIQQQQI7I", b"GSPHSNAP", version, 88, C.sizeof(params_list[0]),
                      len(params_list), n, frames, len(payload), _fnv_words(payload), 0,
                      *([0] * 7))
    assert len(hdr) == 88
    path.write_bytes(hdr + payload)


def test_info_reads_documented_layout(gsph, tmp_path):
    _, p, pos = dam_scene(gsph, n_side=5)
    st = (pos, np.zeros_like(pos), np.zeros_like(pos))
    f = tmp_path / "a.gsnap"
    write_snapshot(f, [p, p], [st, st], frames=42)
    assert gsph.snapshot_info(f) == {"n_scenes": 2, "n_particles": 2 * len(pos), "frames": 42}


def test_info_rejects_foreign_and_inconsistent_files(gsph, tmp_path):
    f = tmp_path / "junk"
    f.write_bytes(b"not a snapshot" * 10)
    with pytest.raises(gsph.GsphError) as ei:
        gsph.snapshot_info(f)
    assert ei.value.status == gsph.ERR_PARSE
    f.write_bytes(b"GSPH")
    with pytest.raises(gsph.GsphError) as ei:
        gsph.snapshot_info(f)
    assert ei.value.status == gsph.ERR_IO
    _, p, pos = dam_scene(gsph, n_side=4)
    st = (pos, np.zeros_like(pos), np.zeros_like(pos))
    write_snapshot(f, [p], [st], version=2)
    with pytest.raises(gsph.GsphError) as ei:
        gsph.snapshot_info(f)
    assert ei.value.status == gsph.ERR_PARSE
    with pytest.raises(gsph.GsphError) as ei:
        gsph.snapshot_info(tmp_path / "missing")
    assert ei.value.status == gsph.ERR_IO
