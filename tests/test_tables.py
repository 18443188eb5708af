"""Plans from host-built tables (fftj_plan_c2c_from_tables): the caller --
FFTJ's Julia planner in a Julia front end -- computes the roots of unity
and the resampling tables, the library only uploads them. Here numpy plays
the host: roots from np.exp, resampling tables from a float64 numpy
restatement of FFTJ's _resample_parts (src/resample.jl:202-256). CPU tests
check the argument validation (it runs before any CUDA call); GPU tests
check the transforms against numpy's FFT and against the library's own
plans."""
import ctypes

import numpy as np
import pytest

from conftest import parity_tol, rel_l2


@pytest.fixture(scope="module")
def F():
    import fftj
    fftj.build()
    return fftj


def roots(N, direction):
    return np.exp(direction * 2j * np.pi * np.arange(N) / N)


def es(z, beta):
    z = np.asarray(z, dtype=np.float64)
    out = np.zeros_like(z)
    inside = np.abs(z) < 1
    out[inside] = np.exp(beta * (np.sqrt(1 - z[inside] ** 2) - 1))
    return out


def resample_tables(orc, T, n, scale):
    m, w, beta = orc.resample_params(T, n)
    h = w // 2
    z, wq = np.polynomial.legendre.leggauss(2 * w + 20)
    pos = z > 0
    j = np.arange(n)
    nu = np.where(j < (n + 1) // 2, j, j - n) / m
    phi = (wq[pos] * es(z[pos], beta) * np.cos(np.pi * np.outer(nu * w, z[pos]))).sum(axis=1)
    corr = scale / (w * phi)
    k = np.arange(n, dtype=np.int64)
    q, rr = (k * m) // n, (k * m) % n
    l0 = (q - h + 1).astype(np.int32)
    delta = rr / n
    wt = es((delta[:, None] + h - 1 - np.arange(w)[None, :]) / h, beta)
    return {"m": m, "w": w, "corr": corr, "wt": wt.ravel(), "l0": l0}


def _call(F, n, omega, N, rs=None, dtype=1):
    h = ctypes.c_void_p()
    om = np.ascontiguousarray(omega, dtype=np.complex128).view(np.float64) if omega is not None else None
    ptr = om.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if om is not None else None
    return F.lib().fftj_plan_c2c_from_tables(ctypes.byref(h), dtype, n, 1, -1, 1.0, ptr, N, rs)


def test_from_tables_argument_checks(F):
    assert _call(F, 64, None, 64) == 1                      # no roots
    assert _call(F, 64, roots(32, -1), 32) == 2             # smooth n takes N = n
    assert _call(F, 10007, roots(20480, -1), 20480) == 1    # non-smooth n without tables
    bad = F.ResampleTables(20479, 16, None, None, None)
    assert _call(F, 10007, roots(20479, -1), 20479, ctypes.byref(bad)) == 1


torch = pytest.importorskip("torch")


@pytest.mark.gpu
@pytest.mark.parametrize("T,n", [(np.float64, 4096), (np.float32, 42525), (np.float64, 1 << 18), (np.float32, 6864)])
def test_from_tables_smooth(F, T, n):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    rng = np.random.default_rng(n)
    x = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
    ct = torch.complex64 if T == np.float32 else torch.complex128
    xd = torch.from_numpy(x).to(ct).cuda()
    p = F.plan_from_tables(T, n, roots(n, -1), batch=2)
    y = p(xd).cpu().numpy()
    ref = np.fft.fft(x, axis=-1)
    assert rel_l2(y, ref) <= parity_tol(T, n)
    own = F.plan_fft(T, n, batch=2)(xd).cpu().numpy()
    assert rel_l2(y, own) <= parity_tol(T, n)
    # the inverse, normalised, from the conjugate roots
    pi = F.plan_from_tables(T, n, roots(n, +1), batch=2, direction=+1, scale=1.0 / n)
    xb = pi(torch.from_numpy(ref).to(ct).cuda()).cpu().numpy()
    assert rel_l2(xb, x) <= 2 * parity_tol(T, n)


@pytest.mark.gpu
@pytest.mark.parametrize("T,n", [(np.float64, 10007), (np.float32, 10007), (np.float64, 3107)])
def test_from_tables_resampled(F, orc, T, n):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    rs = resample_tables(orc, T, n, 1.0)
    rng = np.random.default_rng(n + 1)
    x = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
    ct = torch.complex64 if T == np.float32 else torch.complex128
    p = F.plan_from_tables(T, n, roots(rs["m"], -1), rs, batch=2)
    assert p.info.route == 2 and p.info.resample_m == rs["m"]
    y = p(torch.from_numpy(x).to(ct).cuda()).cpu().numpy()
    assert rel_l2(y, np.fft.fft(x, axis=-1)) <= parity_tol(T, n)
