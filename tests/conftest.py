import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libbte_gb300.so")


@pytest.fixture(scope="session")
def synthetic_xs(tmp_path_factory):
    from boltzmann_gb300.workloads import write_synthetic_lxcat
    return write_synthetic_lxcat(str(tmp_path_factory.mktemp("xs") / "eAr_synthetic.lxcat"))
