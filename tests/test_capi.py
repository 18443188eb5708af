"""C ABI checks that need no GPU: the library builds for sm_103a, loads, exports
every entry point include/fftj.h declares, and rejects bad arguments before
touching CUDA (FFTJ's ArgumentError / DimensionMismatch)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def fftj():
    import fftj as F
    F.build()
    return F


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "fftj.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fftj_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(fftj):
    L = fftj.lib()
    syms = declared_symbols()
    assert "fftj_execute" in syms and len(syms) >= 9
    for s in syms:
        assert hasattr(L, s), s
    assert b"sm_103a" in L.fftj_version()


def test_python_binding_covers_header(fftj):
    assert set(declared_symbols()) == set(fftj.EXPORTS)


def _plan_c2c(fftj, dtype, dims, batch=1, dirn=-1):
    h = ctypes.c_void_p()
    arr = (ctypes.c_int64 * len(dims))(*dims)
    rc = fftj.lib().fftj_plan_c2c(ctypes.byref(h), dtype, len(dims), arr, batch, 0, 0, dirn, 1.0)
    return rc, h


def test_argument_errors(fftj):
    # src/plan.jl:171 — n < 1 is an ArgumentError
    rc, h = _plan_c2c(fftj, 0, [0])
    assert rc == 1 and h.value is None
    assert "positive" in fftj.lib().fftj_last_error_string().decode()
    assert _plan_c2c(fftj, 7, [8])[0] == 1          # bad dtype
    assert _plan_c2c(fftj, 0, [8], dirn=0)[0] == 1  # bad direction
    assert _plan_c2c(fftj, 0, [8], batch=0)[0] == 1
    h = ctypes.c_void_p()
    arr = (ctypes.c_int64 * 1)(16)
    # idist smaller than the transform: DimensionMismatch
    assert fftj.lib().fftj_plan_c2c(ctypes.byref(h), 0, 1, arr, 2, 8, 0, -1, 1.0) == 2
    assert fftj.lib().fftj_execute(None, None, None, None) == 1
    assert fftj.lib().fftj_plan_destroy(None) == 0


def test_python_argument_errors(fftj):
    with pytest.raises(fftj.ArgumentError):
        fftj.plan_fft(np.float64, 0)
    with pytest.raises(fftj.ArgumentError):
        fftj.plan_fft(np.int32, 8)


def test_no_cpu_fallback_in_product():
    """The product package never imports the oracle or torch.fft."""
    pkg = os.path.join(ROOT, "fftj.jl_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cpp", ".cu", ".h")):
                src = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in src.lower() or f == "__init__.py" and "oracle" not in src, f
                assert "torch.fft" not in src, f
                assert "cufft" not in src.lower(), f
