import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
ORACLE_DIR = os.path.join(ROOT, "oracle")
if ORACLE_DIR not in sys.path:
    sys.path.insert(0, ORACLE_DIR)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def vfvm():
    """The package (its directory name is not a Python identifier, so it is loaded
    through __graft_entry__)."""
    import __graft_entry__
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O
