import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA engine")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Build the library, CLI and oracle once per session (no-op when up to date)."""
    from efficientstructuralgraphclusteringongpus_gb300 import build as pkg_build
    from oracle import build as oracle_build

    pkg_build.build()
    oracle_build.build_oracle()
    oracle_build.build_reference()
    yield


def cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
