import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def engine():
    """The built C-ABI library (compiled in-tree on first use)."""
    import nlchains_gb300 as nlc
    nlc.build()
    nlc.lib()
    return nlc


@pytest.fixture(scope="session")
def gpu(engine):
    """The engine on a GPU; fails loudly (no CPU fallback) when no CUDA device answers."""
    try:
        engine.fp64_peak_tflops(ms=5.0)
    except Exception as e:  # pragma: no cover - only on a box without a working GPU
        pytest.fail(f"CUDA engine unusable on this machine: {e}")
    return engine
