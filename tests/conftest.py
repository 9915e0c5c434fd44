import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# The host package lives in a directory whose name is not a Python
# identifier, so it goes on the path and its modules import by name.
sys.path.insert(0, os.path.join(ROOT, "apogee-vm_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: larger CPU cases")
    config.addinivalue_line("markers", "cpu_host: host-side library code that needs no GPU")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib

    return oracle_lib.lib()
