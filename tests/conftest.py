import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
    # temporary test files (scene files, films, variant builds) stay inside the repository
    if not config.option.basetemp:
        config.option.basetemp = os.path.join(ROOT, ".pytest_tmp")


@pytest.fixture(scope="session")
def dev():
    from radiantium_gb300.device import Device
    d = Device(0)
    yield d
    d.close()
