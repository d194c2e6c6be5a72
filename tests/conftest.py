import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "gdistger-re_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def sgns_lib():
    """The built libsgns.so (built on demand; the build cross-compiles without a GPU)."""
    import build as sgns_build
    import sgns

    sgns_build.build()
    return sgns.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build()
    oracle.lib()
    return oracle
