"""The C-ABI library loads and exports every function include/gsph.h declares
(no compute call: this runs without a GPU)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "gsph.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(gsph_\w+)\s*\(", text)
    return sorted(set(n for n in names if not n.endswith("_t")))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ["gsph_create", "gsph_step", "gsph_arrange", "gsph_density",
                     "gsph_force", "gsph_advance", "gsph_benchmark", "gsph_copy_out",
                     "gsph_scene_load_json", "gsph_grid_sort_dev"]:
        assert required in names


def test_library_exports_every_declared_symbol(gsph):
    lib = C.CDLL(str(gsph.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(gsph):
    assert set(declared_functions()) <= set(gsph._SIGS)


def test_field_constants_match_header(gsph):
    text = (ROOT / "include" / "gsph.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    fields = dict(re.findall(r"\bGSPH_(FIELD_\w+)\s*=\s*(\d+)", text))
    assert len(fields) >= 16
    for name, value in fields.items():
        assert getattr(gsph, name) == int(value), name


def test_header_is_c99_and_links(gsph, tmp_path):
    """include/gsph.h compiles as strict C99 with warnings as errors, and a C
    program links against libgsph.so and calls into it (no GPU needed)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "abi.c"
    src.write_text(
        '#include "gsph.h"\n#include <stdio.h>\n'
        "int main(void) {\n"
        "    gsph_tuning t;\n"
        "    if (gsph_tuning_default(&t) != GSPH_OK) return 2;\n"
        '    printf("%d %d %d\\n", (int)sizeof(gsph_block_task), gsph_abi_version(),\n'
        "           t.sparse_total);\n"
        "    return 0;\n}\n")
    lib = gsph.LIB_PATH.parent
    exe = tmp_path / "abi"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                    f"-I{ROOT / 'include'}", str(src), f"-L{lib}", "-lgsph",
                    f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    assert out.split() == ["32", "1", "96"]


def test_struct_sizes(gsph):
    assert C.sizeof(gsph.BlockTask) == 32
    assert gsph.load_library().gsph_abi_version() == 1


def test_scratch_size_query(gsph):
    lib = gsph.load_library()
    small = lib.gsph_grid_sort_scratch_bytes(1000, 4096)
    big = lib.gsph_grid_sort_scratch_bytes(1 << 20, 1 << 20)
    assert 0 < small < big
    assert small % 256 == 0


def test_create_without_device_fails_cleanly(gsph):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    s = gsph.load_scene(gsph.scene_path("dam_break_262k.json"))
    with pytest.raises(gsph.GsphError) as ei:
        gsph.HybridSystem(gsph.scene_path("dam_break_262k.json"))
    assert ei.value.status == gsph.ERR_NO_DEVICE
    assert s.n_blocks == 1
