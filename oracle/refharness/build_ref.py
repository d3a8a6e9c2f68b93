"""Recipe for the reference-kernel harness (test infrastructure only).

Where the reference tree is present (the development container), its CUDA
sources are compiled as they lie — nothing is copied — into one device image,
oracle/_ref/ref_device.cubin, for sm_103a with the reference's own CUDA flags
(--use_fast_math, --extended-lambda, --expt-relaxed-constexpr, headless).
The layout check proves that ref_layout.h matches the reference's argument
types. Wherever the device image exists (it travels with the repository
snapshot; the GPU machine has no reference tree), the host harness ref_harness.cu
is compiled next to it. Outputs go to oracle/_ref/ only (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = ROOT / "oracle" / "_ref"
# The reference tree's src/ directory: GSPH_REFERENCE_SRC, else the
# development container's checkout.
REFERENCE_SRC = Path(os.environ.get("GSPH_REFERENCE_SRC", "/root/reference/src"))
CUBIN = OUT / "ref_device.cubin"
HARNESS = OUT / "ref_harness"
GENCODE = "arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference harness build failed: {' '.join(map(str, cmd))}\n"
                           f"{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps) -> bool:
    return not out.exists() or any(Path(d).stat().st_mtime > out.stat().st_mtime for d in deps)


def build_device_image() -> bool:
    """Compile the reference's sources into the cubin (needs the reference)."""
    if not REFERENCE_SRC.is_dir():
        return False
    OUT.mkdir(parents=True, exist_ok=True)
    shim = OUT / "shim"
    shim.mkdir(exist_ok=True)
    (shim / "windows.h").write_text("/* empty: headless build on Linux */\n")
    flags = ["-std=c++17", "--use_fast_math", "--extended-lambda",
             "--expt-relaxed-constexpr", "-DGSPH_HEADLESS=1",
             f"-I{REFERENCE_SRC}", f"-I{shim}", f"-I{HERE}"]
    if _stale(CUBIN, [HERE / "ref_device.cu"]):
        _run([_nvcc(), *flags, "-arch=sm_103a", "-cubin", "-o", str(CUBIN),
              str(HERE / "ref_device.cu")])
    _run([_nvcc(), *flags, "-arch=sm_103a", "-c", "-o", str(OUT / "layout_check.o"),
          str(HERE / "layout_check.cu")])
    return True


def build_harness() -> bool:
    """Compile the host harness next to an existing device image."""
    if not CUBIN.exists():
        return False
    srcs = [HERE / "ref_harness.cu", HERE / "ref_layout.h", ROOT / "include" / "gsph.h"]
    if _stale(HARNESS, srcs) or not _is_native(HARNESS):
        stubs = Path(_nvcc()).resolve().parent.parent / "lib64" / "stubs"
        _run([_nvcc(), "-std=c++17", "-O2", "-gencode", GENCODE, f"-I{ROOT / 'include'}",
              "-o", str(HARNESS), str(HERE / "ref_harness.cu"), f"-L{stubs}", "-lcuda"])
    return True


def _is_native(path: Path) -> bool:
    """True if the executable was built for this machine's architecture."""
    import platform
    if not path.exists():
        return False
    head = path.read_bytes()[:20]
    if head[:4] != b"\x7fELF":
        return False
    machine = int.from_bytes(head[18:20], "little")
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    return want is None or machine == want


def build_if_available() -> bool:
    build_device_image()
    return build_harness()


if __name__ == "__main__":
    print("device image:", build_device_image(), "harness:", build_harness())
