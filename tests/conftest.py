import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for path in (os.path.join(ROOT, "fpm-rs_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if path not in sys.path:
        sys.path.insert(0, path)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built libfpm_gpu.so")


@pytest.fixture(scope="session")
def native_library():
    import build as native_build

    native_build.build()
    return native_build.LIB


@pytest.fixture(scope="session")
def oracle_module():
    import oracle

    oracle.build()
    return oracle
