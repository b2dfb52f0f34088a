import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (runs through libvcpcuda.so)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def cuda_lib():
    """The in-tree libvcpcuda.so, built if needed; fails loudly if absent."""
    from vcp_gb300.build import build
    build()
    from vcp_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def golden():
    """The golden vectors the reference's own code produced
    (tests/golden/golden.npz, written by tests/golden/make_golden.py)."""
    import numpy as np
    return np.load(ROOT / "tests" / "golden" / "golden.npz")
