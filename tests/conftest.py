import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle.load()


@pytest.fixture(scope="session")
def product_lib():
    from pltfalcor_gb300 import build, capi
    build.build()
    return capi.load_library()


@pytest.fixture(scope="session")
def profiles(product_lib):
    from pltfalcor_gb300 import spectra
    return spectra.standard_profiles(product_lib)
