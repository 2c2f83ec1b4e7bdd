import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_addoption(parser):
    parser.addoption("--runlong", action="store_true", default=False,
                     help="also run the tests marked long (trajectories of several minutes of oracle time)")


def pytest_collection_modifyitems(config, items):
    if config.getoption("--runlong"):
        return
    skip = pytest.mark.skip(reason="long: run with --runlong")
    for item in items:
        if "long" in item.keywords:
            item.add_marker(skip)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library through the C ABI")
    config.addinivalue_line("markers", "slow: long-running parity case")
    config.addinivalue_line("markers", "long: minutes of oracle time; runs only with --runlong")


@pytest.fixture(scope="session")
def oracle32():
    from oracle.binding import Oracle
    return Oracle(np.float32)


@pytest.fixture(scope="session")
def oracle64():
    from oracle.binding import Oracle
    return Oracle(np.float64)


@pytest.fixture(scope="session")
def zqs_lib():
    """The built CUDA library (built on first use; fails loudly without it)."""
    from zq_smokesimulation_gb300 import build, capi
    build.build()
    return capi.load()


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    if den == 0.0:
        return float(num)
    return float(num / den)
