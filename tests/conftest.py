"""Shared test setup: the `gpu` marker, library builds, small helpers."""
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def engine_lib():
    """Builds (if stale) and loads the engine's shared library."""
    from cudancorr_gb300 import build as B
    B.build()
    from cudancorr_gb300 import api
    return api.load_library()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
