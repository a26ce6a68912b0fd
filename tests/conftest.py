"""Test configuration: the ``gpu`` marker and import paths.

``-m "not gpu"`` runs the oracle pins, golden fixtures, host logic and the C-ABI
symbol checks on any machine; ``-m gpu`` runs the parity tests through the C ABI on a
GB300 (the library is built there by ``__graft_entry__.build()``).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "itensornetworksnext.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib_built():
    """Build libitn_gpu.so if needed (nvcc cross-compiles without a GPU)."""
    return load_build_module().build()


def load_build_module():
    """itensornetworksnext.jl_gb300/build.py, loaded by path (no name clash)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("itn_build_recipe", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod
