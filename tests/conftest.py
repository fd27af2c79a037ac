import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # TL_WATCHDOG=<seconds>: dump every thread's Python stack periodically
    # (shows which library call a slow test is in, even inside C code)
    w = os.environ.get("TL_WATCHDOG")
    if w:
        import faulthandler
        faulthandler.dump_traceback_later(float(w), repeat=True)


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden_c1():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "config1.npz")))


@pytest.fixture(scope="session")
def product_lib():
    """Builds bin/liblcirs.so (nvcc, sm_103a) and returns its path."""
    from triplelens_gb300 import build
    build.build()
    return os.path.join(ROOT, "bin", "liblcirs.so")
