import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def eblib():
    from electricbubbles_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def gpu_ctx_factory(eblib):
    from electricbubbles_gb300.api import Context

    made = []

    def make(**kw):
        # the FMM unless a test asks for the small-problem direct sums (test_gpu_direct.py)
        kw.setdefault("direct_max", -1)
        c = Context(**kw)
        made.append(c)
        return c

    yield make
    for c in made:
        c.close()
