"""Build the CUDA library (libgsph.so) and the `gsph` command in-tree.

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked into
lib/libgsph.so; the command links against it with an $ORIGIN rpath. Outputs
stay inside this package directory (lib/ is git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
ROOT = PKG.parent

CUDA_SOURCES = ["grid.cu", "split.cu", "physics.cu", "system.cu", "noalloc.cu"]
CXX_SOURCES = ["scene.cpp", "snapshot.cpp", "server.cpp"]
GENCODE = "arch=compute_103a,code=sm_103a"


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put CUDA on PATH)")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if os.environ.get("GSPH_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose_ptxas: bool = False, force: bool = False) -> Path:
    """Compile libgsph.so and the gsph command; return the library path."""
    nvcc = nvcc_path()
    LIB.mkdir(exist_ok=True)
    objdir = LIB / "obj"
    objdir.mkdir(exist_ok=True)
    headers = [CSRC / "gsph_internal.h", ROOT / "include" / "gsph.h"]
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", f"-I{ROOT / 'include'}"]
    jobs = []
    for src in CUDA_SOURCES:
        obj = objdir / (src + ".o")
        cmd = [nvcc, *common, "-gencode", GENCODE, "-lineinfo", "--use_fast_math",
               "-c", str(CSRC / src), "-o", str(obj)]
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
        jobs.append((obj, cmd, [CSRC / src, *headers]))
    for src in CXX_SOURCES:
        obj = objdir / (src + ".o")
        cmd = [nvcc, *common, "-c", str(CSRC / src), "-o", str(obj)]
        jobs.append((obj, cmd, [CSRC / src, *headers]))
    todo = [(o, c) for o, c, d in jobs if force or verbose_ptxas or _stale(o, d)]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda oc: _run(oc[1]), todo))
    objs = [o for o, _, _ in jobs]
    lib = LIB / "libgsph.so"
    if force or todo or _stale(lib, objs):
        _run([nvcc, "-shared", "-cudart", "static", "-o", str(lib), *map(str, objs)])
    cli = LIB / "gsph"
    if force or _stale(cli, [lib, CSRC / "cli.cpp"]):
        _run(["g++", "-std=c++17", "-O2", str(CSRC / "cli.cpp"), "-o", str(cli),
              f"-L{LIB}", "-lgsph", "-Wl,-rpath,$ORIGIN"])
    return lib


if __name__ == "__main__":
    v = "--ptxas" in sys.argv
    print(build(verbose_ptxas=v, force="--force" in sys.argv))
