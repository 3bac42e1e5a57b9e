"""Test configuration: paths, the `gpu` marker and shared fixtures."""
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
for p in (REPO, REPO / "enblend-enfuse_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libenbgpu.so")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ctx():
    import enbgpu
    from enbgpu import _build
    _build.build()
    c = enbgpu.Context(0)
    yield c
    c.close()
