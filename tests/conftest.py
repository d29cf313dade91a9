import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("", "oracle", "go-melt_gb300"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")
CASES = ("track_const", "phase_powder", "two_layers")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU-only checks")


_cache = {}


def golden(case):
    import stateio

    if case not in _cache:
        _cache[case] = stateio.load(os.path.join(GOLDEN, f"{case}.npz"))
    return _cache[case]


@pytest.fixture(params=CASES)
def case(request):
    return request.param
