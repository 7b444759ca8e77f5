import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); parity tests through the C ABI")


def pytest_collection_modifyitems(config, items):
    """A solve that misses its tolerance warns (RuntimeWarning); in the GPU tests that is an
    error, so a test only passes on converged solves. Tests that expect non-convergence
    catch the warning with pytest.warns."""
    for item in items:
        if item.get_closest_marker("gpu") is not None:
            item.add_marker(pytest.mark.filterwarnings("error::RuntimeWarning"))


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as g
    return g.load_package()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib(pkg):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    import __graft_entry__ as g
    g._load_build_module().build()
    pkg.load()
    return pkg
