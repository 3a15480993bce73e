import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def lib():
    """The built libthc_gb300.so (built on demand; no GPU needed to load it)."""
    from thcpp_gb300 import build, capi
    build.build()
    return capi.load()


_SYS = {}


def system(name):
    """Cached synthetic system by workload name."""
    from thcpp_gb300 import synth
    if name not in _SYS:
        _SYS[name] = synth.config(name)
    return _SYS[name]


@pytest.fixture(scope="session")
def gpu_ctx_fp64(lib):
    from thcpp_gb300 import capi
    with capi.Context(0, capi.THC_PREC_FP64) as c:
        yield c


@pytest.fixture(scope="session")
def gpu_ctx_mixed(lib):
    from thcpp_gb300 import capi
    with capi.Context(0, capi.THC_PREC_MIXED) as c:
        yield c
