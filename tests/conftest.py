"""Shared test set-up: import paths, the `gpu` marker, built artefacts.

Tests marked `gpu` need a CUDA device and the sm_103a library; the others run
on any CPU (they load the library only to check its exports and its host-side
scene/parameter code, which makes no CUDA call).
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG_DIR = ROOT / "fast-general-gpu-sph-framework_gb300"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def load_package():
    """Import the package directory (its name is not a Python identifier)."""
    if "gsph_gb300" in sys.modules:
        return sys.modules["gsph_gb300"]
    spec = importlib.util.spec_from_file_location(
        "gsph_gb300", PKG_DIR / "__init__.py", submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["gsph_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gsph():
    spec = importlib.util.spec_from_file_location("gsph_build", PKG_DIR / "build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    return load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def cuda_device(gsph):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device visible to a test marked gpu")
    return 0
