import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as g
    return g.load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as O  # the CPU restatement (checker)
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu(pkg):
    """The package with its CUDA library loaded (fails loudly if missing)."""
    pkg.build_recipe.build()
    pkg.load()
    return pkg
