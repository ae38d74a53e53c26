"""The C-ABI library: it loads, exports every function include/*.h declares, and
fails loudly (no CPU fallback) where no CUDA device is present."""
import ctypes as C
import os
import re

import pytest

import mrcpp_gb300 as mw
from conftest import has_gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("mwgpu.h", "mwhost.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(mwgpu_\w+|mwh_\w+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_function():
    L = C.CDLL(mw.LIB_PATH)
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_the_abi():
    names = set(declared_functions())
    bound = set(mw._SIGS)
    # every declared function except the allocation-free level call is bound in the package
    assert names - bound <= {"mwgpu_apply_level_static"}, names - bound


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_device_fails_loudly():
    L = mw.lib()
    ctx = C.c_void_p()
    rc = L.mwgpu_init(C.byref(ctx), C.byref(mw.MwgpuConfig()))
    assert rc == 5  # MWGPU_ERR_NO_DEVICE
    assert b"no CUDA device" in L.mwgpu_last_error(None)
    mra = mw.MRA(box=(-20, 20), order=3, basis=mw.INTERPOLATING)
    P = mw.PoissonOperator(mra, 1e-2)
    f = mw.FunctionTree(mra)
    mw.project(1e-2, f, [(1.0, 5.0, (0, 0, 0))])
    with pytest.raises(mw.MWGPUError) as e:
        mw.apply(1e-2, mw.FunctionTree(mra), P, f)
    assert e.value.code == 5


def test_null_arguments_are_rejected():
    L = mw.lib()
    assert L.mwgpu_destroy(None) == 1
    assert L.mwgpu_apply_level(None, None, None, None, None, 0, 1e-3, -1.0, None, None) == 1
    assert L.mwh_apply(1e-3, None, None, None, -1, 0, 0, None) == 1
