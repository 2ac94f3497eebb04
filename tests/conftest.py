import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the native libraries and the oracle once per session."""
    from hspike_gb300.build import build
    from oracle.build_oracle import build as build_oracle

    build()
    build_oracle()


def has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


GOLDEN = os.path.join(ROOT, "tests", "golden")
