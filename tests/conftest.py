"""Test configuration: the ``gpu`` marker and import paths.

``-m "not gpu"`` runs the oracle checks, host logic and ABI-export checks on
CPU; ``-m gpu`` runs the CUDA parity tests through the C ABI."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "exactclosure.jl_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def built_lib():
    """Build libexc.so in-tree if it is missing, then load it."""
    import build as exc_build  # exactclosure.jl_gb300/build.py

    exc_build.build()
    from exactclosure_gb300 import _lib

    return _lib.lib()
