"""The allocation-free entry point, fftj_execute_noalloc_c2c.

It serves callers that cannot allocate device memory at the moment they
transform -- real-time loops that forbid allocation after start-up (an
allocation can block on the driver for an unbounded time), and hosts that own
all device memory through their own pool. Instead of a plan's
workspace it uses one static device array inside the library, so this test
checks, through the C ABI, that its outputs match the plan path
(fftj_plan_c2c + fftj_execute) within the parity tolerance on two calls in a
row, that its size limit is enforced, and that device memory in use does not
grow. This file is named to run last; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from conftest import parity_tol, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CT = {np.float32: torch.complex64, np.float64: torch.complex128}
DT = {np.float32: 0, np.float64: 1}


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import fftj
    fftj.build()
    return fftj.lib()


def plan_result(L, T, n, batch, direction, scale, x):
    h = ctypes.c_void_p()
    dims = (ctypes.c_int64 * 1)(n)
    assert L.fftj_plan_c2c(ctypes.byref(h), DT[T], 1, dims, batch, 0, 0, direction, scale) == 0
    try:
        y = torch.empty_like(x)
        assert L.fftj_execute(h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), None) == 0
        torch.cuda.synchronize()
        return y
    finally:
        L.fftj_plan_destroy(h)


def noalloc(L, T, n, batch, direction, scale, x, y):
    return L.fftj_execute_noalloc_c2c(DT[T], n, batch, direction, scale, ctypes.c_void_p(x.data_ptr()),
                                      ctypes.c_void_p(y.data_ptr()), None)


CASES = [
    (np.float32, 1 << 16, 4, -1, 1.0),        # two passes
    (np.float64, 4096, 3, +1, 1.0 / 4096),    # one pass, normalised inverse
    (np.float32, 42525, 2, -1, 1.0),          # two mixed-radix passes
    (np.float64, 1 << 18, 2, -1, 1.0),        # two passes, F64
]


def test_noalloc_matches_plan_two_calls_in_a_row(lib):
    rng = np.random.default_rng(2024)
    inputs = []
    for T, n, batch, direction, scale in CASES:
        x = torch.from_numpy(rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n)))
        inputs.append(x.to(CT[T]).cuda())
    refs = [plan_result(lib, T, n, b, d, s, x) for (T, n, b, d, s), x in zip(CASES, inputs)]
    # Round 0 warms up: it loads the library's module (which holds the
    # static scratch array) and torch's own kernels used below (zero_, the
    # device-to-host copies). Rounds 1 and 2 are the two calls in a row that
    # are compared with the plan path; device memory in use must not grow
    # across them.
    outs = [torch.empty_like(x) for x in inputs]
    free_before = None
    for rnd in range(3):
        if rnd == 1:
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
        for (T, n, b, d, s), x, y, ref in zip(CASES, inputs, outs, refs):
            y.zero_()
            assert noalloc(lib, T, n, b, d, s, x, y) == 0, lib.fftj_last_error_string()
            torch.cuda.synchronize()
            err = rel_l2(y.cpu().numpy(), ref.cpu().numpy())
            assert err <= parity_tol(T, n), (rnd, T, n, err)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free_before


def test_noalloc_in_place(lib):
    T, n, b = np.float32, 1 << 16, 2
    x = torch.randn(b, n, dtype=CT[T], device="cuda")
    ref = plan_result(lib, T, n, b, -1, 1.0, x)
    z = x.clone()
    assert noalloc(lib, T, n, b, -1, 1.0, z, z) == 0
    torch.cuda.synchronize()
    assert rel_l2(z.cpu().numpy(), ref.cpu().numpy()) <= parity_tol(T, n)


def test_noalloc_limits(lib):
    x = torch.zeros(16, 1 << 20, dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    # 16 * 2^20 * 8 B = 128 MiB > the 63 MiB scratch for the intermediate
    assert noalloc(lib, np.float32, 1 << 20, 16, -1, 1.0, x, y) == 1
    assert b"63 MiB" in lib.fftj_last_error_string()
    # non-smooth and three-pass lengths are not served by this entry point
    assert noalloc(lib, np.float32, 10007, 1, -1, 1.0, x, y) == 5
    assert noalloc(lib, np.float32, 1 << 22, 1, -1, 1.0, x, y) == 5
    assert noalloc(lib, np.float32, 0, 1, -1, 1.0, x, y) == 1
