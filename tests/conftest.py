import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    # the library and the oracle are built in-tree (incremental, seconds)
    from mrcpp_gb300 import build as b

    b.build()
    import oracle

    oracle.build()


def has_gpu():
    try:
        import ctypes

        import mrcpp_gb300 as mw

        ctx = ctypes.c_void_p()
        cfg = mw.MwgpuConfig()
        rc = mw.lib().mwgpu_init(ctypes.byref(ctx), ctypes.byref(cfg))
        if rc == 0:
            mw.lib().mwgpu_destroy(ctx)
        return rc == 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not has_gpu():
        pytest.fail("a CUDA device is required for tests marked gpu")
    return True
