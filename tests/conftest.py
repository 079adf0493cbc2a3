import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))

    return load


@pytest.fixture(scope="session")
def built_lib():
    from moquimc_gb300 import build

    build.build_library()
    from moquimc_gb300 import capi

    return capi.load()


@pytest.fixture(scope="session")
def oracle():
    import mqo

    mqo.lib()
    return mqo


@pytest.fixture(scope="session")
def gpu_ctx_factory(built_lib):
    from moquimc_gb300 import capi

    made = []

    def make():
        c = capi.Context(0)
        made.append(c)
        return c

    yield make
    for c in made:
        c.close()
