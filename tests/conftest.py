import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpnjl_cuda.so")


@pytest.fixture(scope="session")
def engine_factory():
    """Create GapEngine contexts on cuda:0 (GPU tests only); closed at session end."""
    from julia_relaxtime_gb300.engine import GapEngine

    made = []

    def make(p_num=64, t_num=8):
        e = GapEngine(device=0, p_num=p_num, t_num=t_num)
        made.append(e)
        return e

    yield make
    for e in made:
        e.close()
