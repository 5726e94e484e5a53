import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA engine)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the engine and the oracle in-tree once per session."""
    from spike_gb300 import _build
    _build.build_engine()
    _build.build_oracle()


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
