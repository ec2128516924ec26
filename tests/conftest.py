import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C-ABI library")


@pytest.fixture(scope="session")
def lp_lib():
    from pdal_gb300 import _native as N
    from pdal_gb300 import build

    if not N.lib_path("libcp_al_gb300.so").exists():
        build.build_product()
    return N.load_lp()


@pytest.fixture(scope="session")
def qp_lib():
    from pdal_gb300 import _native as N
    from pdal_gb300 import build

    if not N.lib_path("libfa_cp_gb300.so").exists():
        build.build_product()
    return N.load_qp()
