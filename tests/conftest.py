"""Shared pytest setup: import paths and the ``gpu`` marker."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "permutationalinvariantdynamics.jl_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib_built():
    """Builds libpicuda.so in-tree once per session (nvcc cross-compiles without a GPU)."""
    sys.path.insert(0, str(PKG))
    import build_lib
    return build_lib.build()
