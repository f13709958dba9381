import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
TESTS = Path(__file__).resolve().parent
for p in (str(ROOT), str(TESTS)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = TESTS / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers",
                            "gpu: needs a CUDA GPU (runs the CUDA engine)")


@pytest.fixture(scope="session")
def built():
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def port(built):
    from oracle import pyoracle
    return pyoracle.port()


@pytest.fixture(scope="session")
def ref(built):
    from oracle import pyoracle
    r = pyoracle.ref()
    if r is None:
        pytest.skip("reference sources not present (fixtures cover this)")
    return r


def golden(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))
