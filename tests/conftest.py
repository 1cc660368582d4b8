"""Shared fixtures.  GPU tests carry @pytest.mark.gpu and call the CUDA path
through the C ABI; everything else runs on the CPU."""
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as ge  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the CUDA path")


@pytest.fixture(scope="session")
def pkg():
    return ge.load_package()


@pytest.fixture(scope="session")
def ora():
    m = ge.load_oracle()
    m.build()
    return m


@pytest.fixture(scope="session")
def gpu(pkg):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    pkg.build()
    pkg.lib()
    torch.cuda.set_device(0)
    return pkg
