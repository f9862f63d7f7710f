import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
for p in (REPO, REPO / "spin-tracking_gb300", REPO / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = REPO / "tests" / "golden"
GOLDEN_CASES = sorted(p.stem for p in GOLDEN.glob("*.bin"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from _oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def stlib():
    """The engine's C ABI library (built in-tree if missing; loading needs no GPU)."""
    from spintrack import _capi
    return _capi.load(build_if_missing=True)


@pytest.fixture(scope="session")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from spintrack import _capi
    _capi.load(build_if_missing=True)
    return torch.device("cuda:0")
