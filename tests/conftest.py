import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Native library and oracle are built in-tree once per session (no-ops when up to date)."""
    from dumbray_gb300 import build as native
    native.build()
    import _oracle
    _oracle.oracle()
    yield


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
