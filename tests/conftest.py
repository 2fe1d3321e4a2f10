import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import dg_oracle

    dg_oracle.build()
    return dg_oracle


@pytest.fixture(scope="session")
def ctx():
    import dendro_gb300

    return dendro_gb300.default_context()
