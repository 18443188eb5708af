"""GPU parity: the sm_103a path (through the C ABI) against the oracle (the
FFTJ CPU restatement in the config dtype) and FP64 references.

Bar: relative L2 error <= 5 * log2(N) * eps(T) against both the oracle and
the FP64 reference (the parity bar of the task; tighter than the reference
suite's 50/100/200 eps classes for N >= 2^10). Full-size configs are checked
on sampled batches against the oracle and on every batch through
size-independent properties (inverse round trip, Parseval, exact FP64 bins).
"""
import ctypes

import numpy as np
import pytest

from conftest import EPS, parity_tol, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

T_LIST = [np.float32, np.float64]
CT = {np.float32: torch.complex64, np.float64: torch.complex128}
RT = {np.float32: torch.float32, np.float64: torch.float64}


@pytest.fixture(scope="module")
def fftj():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import fftj as F
    F.build()
    return F


def dev(x, T):
    t = torch.from_numpy(np.ascontiguousarray(x))
    t = t.to(CT[T] if np.iscomplexobj(x) else RT[T])
    return t.cuda()


def host(t):
    return t.cpu().numpy()


def cn(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def _sizes(golden, prefix):
    return sorted(int(k[len(prefix):]) for k in golden.files if k.startswith(prefix))


# --------------------------------------------------------------------------
# reference test-suite sizes (test/runtests.jl) against golden and oracle


@pytest.mark.parametrize("T", T_LIST)
def test_c2c_reference_sizes(fftj, golden, orc, T):
    for n in _sizes(golden, "c2c_x_"):
        x = golden["c2c_x_%d" % n]
        ref = golden["c2c_y_%d" % n]
        xd = dev(x, T)
        y = host(fftj.plan_fft(T, n)(xd))
        tol = parity_tol(T, n)
        assert rel_l2(y, ref) <= tol, (n, rel_l2(y, ref) / EPS[T])
        yo = orc.Plan1D(T, n, "fft")(x)
        assert rel_l2(y, yo) <= tol, (n, "vs oracle", rel_l2(y, yo) / EPS[T])
        # inverse round trip (runtests.jl:23) and bfft = n * ifft (:76)
        xi = host(fftj.plan_ifft(T, n)(dev(y, T)))
        assert rel_l2(xi, x) <= 2 * tol, n
        xb = host(fftj.plan_bfft(T, n)(dev(ref, T)))
        assert rel_l2(xb, n * x) <= 2 * tol, n


@pytest.mark.parametrize("T", T_LIST)
def test_known_answers(fftj, golden, T):
    for key in golden.files:
        if not key.startswith("kat_"):
            continue
        n = int(key.rsplit("_", 1)[1])
        y = host(fftj.plan_fft(T, n)(dev(golden[key], T)))
        if "impulse" in key:
            assert np.allclose(y, np.ones(n), atol=10 * EPS[T])
        elif n > 3:
            exp = np.zeros(n, dtype=np.complex128)
            exp[3] = n
            assert rel_l2(y, exp) <= parity_tol(T, n), key


@pytest.mark.parametrize("T", T_LIST)
def test_real_reference_sizes(fftj, golden, orc, T):
    for n in _sizes(golden, "r2c_x_"):
        x = golden["r2c_x_%d" % n]
        ref = golden["r2c_y_%d" % n]
        Y = fftj.plan_rfft(T, n)(dev(x, T))
        assert tuple(Y.shape) == (n // 2 + 1,)
        tol = max(parity_tol(T, n), 5 * EPS[T])
        assert rel_l2(host(Y), ref) <= tol, n
        yo = orc.PlanReal(T, n, "rfft")(x)
        assert rel_l2(host(Y), yo) <= 2 * tol, (n, "vs oracle")
        xr = host(fftj.plan_irfft(T, n)(dev(ref, T)))
        assert rel_l2(xr, x) <= 2 * tol, n
        xb = host(fftj.plan_brfft(T, n)(dev(ref, T)))
        assert rel_l2(xb, n * x) <= 2 * tol, n


@pytest.mark.parametrize("T", T_LIST)
def test_nd_reference_shapes(fftj, golden, orc, T):
    for key in golden.files:
        if not key.startswith("nd_x_"):
            continue
        dims = [int(v) for v in key[5:].split("x")]
        n = int(np.prod(dims))
        tol = 200 * EPS[T]
        x = golden[key]
        ref = golden["nd_y_" + key[5:]]
        y = host(fftj.fft(dev(x, T)))
        assert rel_l2(y, ref) <= tol, dims
        assert rel_l2(y, orc.PlanND(T, dims, "fft")(x)) <= tol, dims
        assert rel_l2(host(fftj.ifft(dev(ref, T))), x) <= tol, dims
        xr = golden["ndr_x_" + key[5:]]
        rref = golden["ndr_y_" + key[5:]]
        Y = fftj.rfft(dev(xr, T))
        assert tuple(Y.shape) == rref.shape and rel_l2(host(Y), rref) <= tol, dims
        # the oracle's real N-d plans (batched real edge where FFTJ batches it)
        assert rel_l2(host(Y), orc.PlanND(T, dims, "rfft")(xr)) <= tol, dims
        xi = host(fftj.irfft(dev(rref, T), dims[0]))
        assert rel_l2(xi, xr) <= tol, dims
        assert rel_l2(xi, orc.PlanND(T, dims, "irfft")(rref)) <= tol, dims
        xb = host(fftj.brfft(dev(rref, T), dims[0]))
        assert rel_l2(xb, n * xr) <= tol, dims
        assert rel_l2(xb, orc.PlanND(T, dims, "brfft")(rref)) <= tol, dims


@pytest.mark.parametrize("T", T_LIST)
@pytest.mark.parametrize("shape", [(17, 16), (16, 17), (19, 23), (3, 17, 8), (101, 64), (7, 97)])
def test_nd_nonsmooth_dims(fftj, orc, T, shape):
    """N-d shapes with non-smooth dimensions (batched resampling along the
    axis, FFTJ RsPass), complex and real, against FP64 and the oracle."""
    rng = np.random.default_rng(list(shape))
    x = cn(rng, shape)
    tol = 200 * EPS[T]
    y = host(fftj.fft(dev(x, T)))
    assert rel_l2(y, np.fft.fftn(x)) <= tol, shape
    assert rel_l2(y, orc.PlanND(T, list(reversed(shape)), "fft")(x)) <= tol, shape
    assert rel_l2(host(fftj.ifft(dev(y, T))), x) <= tol, shape
    xr = rng.standard_normal(shape)
    Y = fftj.rfft(dev(xr, T))
    assert rel_l2(host(Y), np.fft.rfftn(xr)) <= tol, shape
    assert rel_l2(host(Y), orc.PlanND(T, list(reversed(shape)), "rfft")(xr)) <= tol, shape
    xi = host(fftj.irfft(Y, shape[-1]))
    assert rel_l2(xi, xr) <= tol, shape
    assert rel_l2(xi, orc.PlanND(T, list(reversed(shape)), "irfft")(host(Y))) <= tol, shape


# --------------------------------------------------------------------------
# the benchmark configurations at full size


def test_config_c64_2e16_batch64(fftj, orc):
    """Plain 1-D forward ComplexF64 FFT, N=2^16, batch 64, U[-1,1) re/im,
    compared to the FFTJ CPU plan (oracle) and FP64 pocketfft."""
    n, B = 1 << 16, 64
    rng = np.random.default_rng(0xF17)
    x = rng.uniform(-1, 1, (B, n)) + 1j * rng.uniform(-1, 1, (B, n))
    y = host(fftj.plan_fft(np.float64, n, batch=B)(dev(x, np.float64)))
    tol = parity_tol(np.float64, n)
    assert rel_l2(y, orc.Plan1D(np.float64, n, "fft")(x)) <= tol
    assert rel_l2(y, np.fft.fft(x, axis=-1)) <= tol


@pytest.mark.parametrize("T", T_LIST)
@pytest.mark.parametrize("n", [42525, 10007, 1 << 18])
def test_config_mixed_prime_batch128(fftj, orc, T, n):
    """ComplexF32/F64 at N = 42525 (3^5 5^2 7), 10007 (prime: resampled) and
    2^18, batch 128, iid standard complex normal: all batches against FP64,
    four sampled batches against the oracle, forward+inverse round trip."""
    B = 128
    rng = np.random.default_rng([0xC0F1, n])
    x = cn(rng, (B, n))
    xd = dev(x, T)
    y = fftj.plan_fft(T, n, batch=B)(xd)
    yh = host(y)
    tol = parity_tol(T, n)
    assert rel_l2(yh, np.fft.fft(x, axis=-1)) <= tol
    pick = [0, 1, 63, 127]
    assert rel_l2(yh[pick], orc.Plan1D(T, n, "fft")(x[pick])) <= tol
    xi = host(fftj.plan_ifft(T, n, batch=B)(y))
    assert rel_l2(xi, x) <= 2 * tol


def _dft_bins(x, ks, sign=-1):
    """Exact-ish FP64 DFT bins X[k] of a long vector (numpy, float64)."""
    n = x.shape[-1]
    j = np.arange(n, dtype=np.int64)
    out = []
    for k in ks:
        e = (j * int(k)) % n
        w = np.exp(sign * 2j * np.pi * e / n)
        out.append(np.dot(x.astype(np.complex128), w))
    return np.array(out)


@pytest.mark.parametrize("T,logn", [(np.float32, 26), (np.float64, 24)])
def test_config_large_single(fftj, T, logn):
    """Single ComplexF32 2^26 / ComplexF64 2^24 (U[-1,1)): the whole output
    vector against FP64 numpy, exact FP64 DFT bins, Parseval, inverse round
    trip."""
    n = 1 << logn
    rng = np.random.default_rng(logn)
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64 if T == np.float32 else np.complex128)
    xd = dev(x, T)
    y = fftj.plan_fft(T, n)(xd)
    yh = host(y)
    ks = [0, 1, 7, n // 3, n // 2, n - 1, 12345, n // 2 + 17]
    ref = _dft_bins(x, ks)
    # per-bin error relative to the rms bin magnitude (sqrt(n) * rms(x))
    scale = np.sqrt(n) * np.sqrt(np.mean(np.abs(x.astype(np.complex128)) ** 2))
    assert np.max(np.abs(yh[ks] - ref)) / scale <= 4 * parity_tol(T, n)
    # Parseval
    px = np.sum(np.abs(x.astype(np.complex128)) ** 2) * n
    py = np.sum(np.abs(yh.astype(np.complex128)) ** 2)
    assert abs(py - px) / px <= parity_tol(T, n)
    # full vector vs FP64 (numpy pocketfft in complex128)
    full = np.fft.fft(x.astype(np.complex128))
    assert rel_l2(yh, full) <= parity_tol(T, n), rel_l2(yh, full) / EPS[T]
    del full
    xi = host(fftj.plan_ifft(T, n)(y))
    assert rel_l2(xi, x) <= 2 * parity_tol(T, n)


def test_config_rfft_2e25_batch4(fftj):
    """Float32 rfft / irfft N=2^25, batch 4, U[-1,1)."""
    n, B = 1 << 25, 4
    rng = np.random.default_rng(25)
    x = rng.uniform(-1, 1, (B, n)).astype(np.float32)
    Y = fftj.plan_rfft(np.float32, n, batch=B)(dev(x, np.float32))
    assert tuple(Y.shape) == (B, n // 2 + 1)
    Yh = host(Y)
    tol = parity_tol(np.float32, n)
    ks = [0, 1, 5, n // 4, n // 2, 999]
    for b in (0, 3):
        ref = _dft_bins(x[b], ks)
        scale = np.sqrt(n) * np.sqrt(np.mean(x[b].astype(np.float64) ** 2))
        assert np.max(np.abs(Yh[b, ks] - ref)) / scale <= 4 * tol
    xr = host(fftj.plan_irfft(np.float32, n, batch=B)(Y))
    assert rel_l2(xr, x) <= 2 * tol


def _stress(rng, shape):
    x = cn(rng, shape)
    flat = x.reshape(-1)
    idx = rng.choice(flat.size, size=flat.size // 100, replace=False)
    flat[idx] *= 1e3
    return x


def test_config_precision_2e20_batch64(fftj):
    """ComplexF32 2^20, batch 64, standard complex normal with 1% of entries
    x1e3: plain FP32 form against the FP64 reference."""
    n, B = 1 << 20, 64
    rng = np.random.default_rng(20)
    x = _stress(rng, (B, n)).astype(np.complex64)
    y = host(fftj.plan_fft(np.float32, n, batch=B)(dev(x, np.float32)))
    pick = [0, 31, 63]
    ref = np.fft.fft(x[pick].astype(np.complex128), axis=-1)
    assert rel_l2(y[pick], ref) <= parity_tol(np.float32, n)


def test_config_precision_2d_4096(fftj, orc):
    """ComplexF32 2-D 4096x4096 with the 1% x1e3 stress entries."""
    rng = np.random.default_rng(4096)
    x = _stress(rng, (4096, 4096)).astype(np.complex64)
    y = host(fftj.fft(dev(x, np.float32)))
    ref = np.fft.fft2(x.astype(np.complex128))
    assert rel_l2(y, ref) <= parity_tol(np.float32, 4096 * 4096)
    # the FFTJ CPU plan of this shape: NdPlan run through Fs2Plan
    po = orc.PlanND(np.float32, [4096, 4096], "fft")
    assert po.route == "Fs2Plan"
    yo = po(x)
    assert rel_l2(y, yo) <= parity_tol(np.float32, 4096 * 4096)
    # two HBM sweeps on request, as FFTJ's Fs2Plan (src/fourstep.jl:500-552):
    # the contiguous rows, then the strided 4096-point columns in one pass
    p2 = fftj.Plan(np.float32, (4096, 4096), kind="c2c", opts={"wide_axis": 1})
    inf = p2.info
    assert inf.npasses == 2 and list(inf.pass_radix[:2]) == [4096, 4096]
    assert list(inf.pass_threads[:2])[1] == 1024 and inf.specialized_passes == 2
    y2 = host(p2(dev(x, np.float32)))
    assert rel_l2(y2, ref) <= parity_tol(np.float32, 4096 * 4096)
    assert rel_l2(y2, yo) <= parity_tol(np.float32, 4096 * 4096)


@pytest.mark.parametrize("shape", [(4096, 64), (4096, 3, 4), (2, 4096, 12), (4096, 6)])
def test_strided_4096_axis_one_pass(fftj, orc, shape):
    """opts.wide_axis: strided ComplexF32 axes of length 4096 (one pass of
    4-column tiles when the inner extent is a multiple of 4, else two
    passes), forward and inverse, against FP64 numpy and the oracle's N-d
    plan."""
    rng = np.random.default_rng(list(shape))
    x = cn(rng, shape).astype(np.complex64)
    tol = parity_tol(np.float32, int(np.prod(shape)))
    dims = tuple(reversed(shape))
    pf = fftj.Plan(np.float32, dims, kind="c2c", opts={"wide_axis": 1})
    pb = fftj.Plan(np.float32, dims, kind="c2c", direction=1, scale=1.0 / x.size, opts={"wide_axis": 1})
    y = host(pf(dev(x, np.float32)))
    assert rel_l2(y, np.fft.fftn(x.astype(np.complex128))) <= tol, shape
    assert rel_l2(y, orc.PlanND(np.float32, list(dims), "fft")(x)) <= tol, shape
    assert rel_l2(host(pb(dev(y, np.float32))), x) <= tol, shape
    inner = int(np.prod(shape[shape.index(4096) + 1:]))
    for p in (pf, pb):
        inf = p.info
        assert (4096 in list(inf.pass_radix[:inf.npasses])) == (inner % 4 == 0), shape


def test_config_rfft3d_256(fftj):
    """Float32 256^3 3-D rfft (and its irfft) against FP64 numpy."""
    rng = np.random.default_rng(256)
    x = rng.standard_normal((256, 256, 256)).astype(np.float32)
    Y = fftj.rfft(dev(x, np.float32))
    assert tuple(Y.shape) == (256, 256, 129)
    ref = np.fft.rfftn(x.astype(np.float64))
    tol = parity_tol(np.float32, 256 ** 3)
    assert rel_l2(host(Y), ref) <= tol
    assert rel_l2(host(fftj.irfft(Y, 256)), x) <= 2 * tol


# --------------------------------------------------------------------------
# API idioms (test/runtests.jl:264-328), in-place, strides, streams


@pytest.mark.parametrize("T", T_LIST)
@pytest.mark.parametrize("n", [96, 11])
def test_api_idioms(fftj, T, n):
    rng = np.random.default_rng(0xC0A7)
    x = cn(rng, n)
    xr = rng.standard_normal(n)
    tol = 100 * EPS[T]
    xd = dev(x, T)
    p = fftj.plan_fft(xd, flags="ignored")
    assert rel_l2(host(p * xd), np.fft.fft(x)) <= tol
    y = torch.empty_like(xd)
    assert fftj.mul_(y, p, xd) is y
    assert rel_l2(host(y), np.fft.fft(x)) <= tol
    assert rel_l2(host(fftj.plan_bfft(xd) * xd), n * np.fft.ifft(x)) <= tol
    # in place: DSP's p! * buf; inv(p!).p
    pin = fftj.plan_fft_(xd)
    z = xd.clone()
    assert (pin * z) is z
    assert rel_l2(host(z), np.fft.fft(x)) <= tol
    ip = fftj.inv(pin).p
    assert (ip * z) is z
    assert rel_l2(host(z), n * x) <= tol
    z2 = xd.clone()
    pin * z2
    fftj.inv(pin) * z2
    assert rel_l2(host(z2), x) <= tol
    # rfft / brfft (DSP _fftfilt!)
    xrd = dev(xr, T)
    pr = fftj.plan_rfft(xrd)
    X = pr * xrd
    assert rel_l2(host(X), np.fft.rfft(xr)) <= tol
    pbr = fftj.plan_brfft(X, n)
    assert rel_l2(host(pbr * X), n * np.fft.irfft(np.fft.rfft(xr), n)) <= tol
    # one-shots
    assert rel_l2(host(fftj.fft(xd)), np.fft.fft(x)) <= tol
    assert rel_l2(host(fftj.ifft(xd)), np.fft.ifft(x)) <= tol
    assert rel_l2(host(fftj.bfft(xd)), n * np.fft.ifft(x)) <= tol
    assert rel_l2(host(fftj.rfft(xrd)), np.fft.rfft(xr)) <= tol
    assert rel_l2(host(fftj.irfft(X, n)), xr) <= tol
    assert rel_l2(host(fftj.fft_(xd.clone())), np.fft.fft(x)) <= tol
    assert fftj.size(p) == (n,) and fftj.size(pbr) == (n // 2 + 1,)
    # region validation and DimensionMismatch (runtests.jl:327, 426)
    with pytest.raises(fftj.ArgumentError):
        fftj.plan_fft(xd, 2)
    with pytest.raises(fftj.DimensionMismatch):
        p(torch.zeros(n + 1, dtype=CT[T], device="cuda"))
    with pytest.raises(fftj.ArgumentError):
        p(torch.zeros(n, dtype=CT[T]))  # host tensor: there is no CPU path


@pytest.mark.parametrize("T", T_LIST)
def test_inplace_and_determinism(fftj, T):
    rng = np.random.default_rng(7)
    for n, B in ((4096, 8), (42525, 3), (1 << 18, 2), (10007, 4)):
        x = dev(cn(rng, (B, n)), T)
        p = fftj.plan_fft(T, n, batch=B)
        y1 = p(x)
        y2 = p(x)
        assert torch.equal(y1, y2), n  # bitwise run-to-run
        z = x.clone()
        p(z, z)
        assert torch.equal(z, y1), n   # in == out


@pytest.mark.parametrize("T,n,B,idist,odist", [
    (np.float32, 1000, 5, 1024, 1100),
    (np.float64, 16 * 509, 3, 16 * 509 + 8, 16 * 509 + 24),   # CompositePlan (HvPass lanes)
    (np.float64, 32 * 131, 3, 32 * 131 + 3, 32 * 131 + 5),    # CompositePlan (RsPass lanes)
    (np.float64, 2 * 10007, 2, 2 * 10007 + 2, 2 * 10007 + 6),  # SplitPlan
    (np.float64, 10007, 3, 10010, 10016),                      # HvdhPlan
])
def test_strided_batches_c_abi(fftj, T, n, B, idist, odist):
    """idist/odist > n through the C ABI (padded rows), on the smooth,
    composite, split and Gaussian-resampling routes."""
    L = fftj.lib()
    rng = np.random.default_rng([3, n])
    x = cn(rng, (B, idist)).astype(np.complex64 if T is np.float32 else np.complex128)
    xd = dev(x, T)
    yd = torch.zeros((B, odist), dtype=CT[T], device="cuda")
    h = ctypes.c_void_p()
    dims = (ctypes.c_int64 * 1)(n)
    dt = 0 if T is np.float32 else 1
    assert L.fftj_plan_c2c(ctypes.byref(h), dt, 1, dims, B, idist, odist, -1, 1.0) == 0
    try:
        assert L.fftj_execute(h, ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(yd.data_ptr()), None) == 0
        torch.cuda.synchronize()
        y = host(yd)
        assert rel_l2(y[:, :n], np.fft.fft(x[:, :n], axis=-1)) <= parity_tol(T, n)
        assert np.all(y[:, n:] == 0)
    finally:
        L.fftj_plan_destroy(h)


def test_nondefault_stream(fftj):
    rng = np.random.default_rng(11)
    n, B = 1 << 16, 16
    x = dev(cn(rng, (B, n)), np.float32)
    p = fftj.plan_fft(np.float32, n, batch=B)
    ref = p(x)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        y = p(x)
    s.synchronize()
    assert torch.equal(y, ref)


def test_library_loaded_from_tree(fftj):
    import os
    assert os.path.dirname(fftj._build.LIB).endswith("fftj.jl_gb300")
    assert fftj.lib()._name == fftj._build.LIB


# --------------------------------------------------------------------------
# Gaussian resampling (HvdH, src/hvdh.jl): FFTJ's route for odd non-smooth
# n >= 1000 (F64) / >= 16384 (F32) (test/runtests.jl:110-144, 411-414)


@pytest.mark.parametrize("T,n", [(np.float64, 3107), (np.float64, 10007), (np.float64, 20011),
                                 (np.float64, 65537), (np.float32, 20011), (np.float32, 65537)])
def test_hvdh_route_and_parity(fftj, orc, T, n):
    rng = np.random.default_rng([0x4D4, n])
    B = 3
    x = cn(rng, (B, n))
    p = fftj.plan_fft(T, n, batch=B)
    assert p.route == "HvdhPlan"
    y = p(dev(x, T))
    tol = parity_tol(T, n)
    ref = np.fft.fft(x, axis=-1)
    assert rel_l2(host(y), ref) <= tol, (n, rel_l2(host(y), ref) / EPS[T])
    po = orc.Plan1D(T, n, "fft")
    assert po.route == "HvdhPlan"  # the oracle's HvdH restatement (src/hvdh.jl)
    assert rel_l2(host(y)[:1], po(x[:1])) <= tol
    xi = host(fftj.plan_ifft(T, n, batch=B)(y))
    assert rel_l2(xi, x) <= 2 * tol
    xb = host(fftj.plan_bfft(T, n, batch=B)(dev(ref, T)))
    assert rel_l2(xb, n * x) <= 2 * tol


def test_resample_routes(fftj):
    """Non-smooth lengths below the HvdH thresholds, and even ones, resample
    (test/runtests.jl:412-416)."""
    assert fftj.plan_fft(np.float64, 10006).route == "ResamplePlan"
    assert fftj.plan_fft(np.float32, 10007).route == "ResamplePlan"
    assert fftj.plan_fft(np.float64, 997).route == "ResamplePlan"


@pytest.mark.parametrize("T", T_LIST)
@pytest.mark.parametrize("n", [3969, 6864, 3696, 7150, 3549, 6237, 9 * 11 * 13 * 7])
def test_odd_radix_lengths_that_need_two_passes(fftj, orc, T, n):
    """Lengths whose odd radices need more threads per column than one CTA
    has (e.g. 3969 = 3^4 7^2) run as two passes; forward, inverse and the
    oracle agree."""
    rng = np.random.default_rng(n)
    x = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
    y = host(fftj.plan_fft(T, n, batch=2)(dev(x, T)))
    ref = np.fft.fft(x, axis=-1)
    assert rel_l2(y, ref) <= parity_tol(T, n), (n, rel_l2(y, ref) / EPS[T])
    yo = orc.Plan1D(T, n, "fft")(x[0])
    assert rel_l2(y[0], yo) <= parity_tol(T, n)
    xi = host(fftj.plan_ifft(T, n, batch=2)(dev(y, T)))
    assert rel_l2(xi, x) <= 2 * parity_tol(T, n)


@pytest.mark.parametrize("T,n,B", [(np.float64, 2 * 10007, 2), (np.float64, 6 * 3001, 3),
                                   (np.float32, 4 * 32771, 2)])
def test_split_route(fftj, orc, T, n, B):
    """Even non-smooth lengths n = s p with a small 7-smooth part (s < 16,
    p odd and Gaussian-resampled; FFTJ SplitPlan): decimation, s HvdH
    sub-transforms with the w_n^(r k1) twiddles in their banded solve,
    length-s passes along r. Forward against FP64 numpy and the oracle's
    SplitPlan, normalised inverse round trip."""
    p = fftj.plan_fft(T, n, batch=B)
    assert p.route == "SplitPlan", p.route
    rng = np.random.default_rng(n)
    x = rng.standard_normal((B, n)) + 1j * rng.standard_normal((B, n))
    y = p(dev(x, T))
    tol = parity_tol(T, n)
    assert rel_l2(host(y), np.fft.fft(x, axis=-1)) <= tol
    po = orc.Plan1D(T, n, "fft")
    assert po.route == "SplitPlan", po.route
    assert rel_l2(host(y).reshape(B, n)[:1], po(x[:1])) <= tol
    xi = host(fftj.plan_ifft(T, n, batch=B)(y))
    assert rel_l2(xi, x) <= 2 * tol


@pytest.mark.parametrize("T,n,B", [(np.float64, 16 * 509, 4), (np.float64, 27 * 509, 2), (np.float64, 30 * 4099, 1),
                                   (np.float64, 1024 * 1009, 1), (np.float64, 32 * 131, 3),
                                   (np.float32, 64 * 1031, 2), (np.float32, 256 * 257, 2)])
def test_composite_route(fftj, orc, T, n, B):
    """FFTJ's CompositePlan lengths (7-smooth part s >= 16, src/composite.jl:
    10-101): s-part passes along p lanes, the twiddled transpose, the odd part
    p along rows of s lanes by the batched HvPass (p >= 500) or RsPass.
    Forward against FP64 numpy and the oracle's CompositePlan, normalised
    inverse round trip, both solve factor forms for HvPass."""
    p = fftj.plan_fft(T, n, batch=B)
    assert p.route == "CompositePlan", p.route
    rng = np.random.default_rng([n, 6])
    x = rng.standard_normal((B, n)) + 1j * rng.standard_normal((B, n))
    y = p(dev(x, T))
    tol = parity_tol(T, n)
    assert rel_l2(host(y), np.fft.fft(x, axis=-1)) <= tol
    po = orc.Plan1D(T, n, "fft")
    assert po.route == "CompositePlan", po.route
    assert rel_l2(host(y).reshape(B, n)[:2], po(x[:2])) <= tol
    xi = host(fftj.plan_ifft(T, n, batch=B)(y))
    assert rel_l2(xi, x) <= 2 * tol
    if n // 1024 >= 500 or n in (16 * 509, 27 * 509, 30 * 4099, 64 * 1031):
        pf = fftj.Plan(T, (n,), kind="c2c", batch=B, opts={"hvdh_factors": 2})
        assert pf.route == "CompositePlan"
        assert rel_l2(host(pf(dev(x, T))), host(y)) <= tol


@pytest.mark.parametrize("T", T_LIST)
@pytest.mark.parametrize("n", [16 * 509, 3 * 1009, 12 * 97])
def test_composite_forced(fftj, orc, T, n):
    """opts.route = 4: CompositePlan below FFTJ's size thresholds (odd and
    small smooth parts, HvPass and RsPass), against the oracle's
    FFTJ._composite restatement and FP64 numpy, both directions."""
    B = 3
    rng = np.random.default_rng([n, 4])
    x = cn(rng, (B, n))
    tol = parity_tol(T, n)
    pf = fftj.Plan(T, (n,), kind="c2c", batch=B, opts={"route": 4})
    assert pf.route == "CompositePlan"
    y = host(pf(dev(x, T)))
    assert rel_l2(y, np.fft.fft(x, axis=-1)) <= tol
    assert rel_l2(y, orc.PlanDirect(T, n, "composite")(x)) <= tol
    pb = fftj.Plan(T, (n,), kind="c2c", batch=B, direction=1, scale=1.0 / n, opts={"route": 4})
    assert rel_l2(host(pb(dev(y, T))), x) <= 2 * tol


# FFTJ's HvdH test sizes (test/runtests.jl:110-137), the route forced to
# full-length Gaussian resampling (opts.route = 3, as the reference's tests
# build FFTJ._hvdh directly): tiny and even lengths, halos wider than t.
HVDH_FORCED = [11, 13, 17, 19, 22, 23, 26, 34, 38, 46, 97, 101, 202, 331, 997, 1001]


@pytest.mark.parametrize("T", T_LIST)
def test_hvdh_forced_reference_sizes(fftj, orc, T):
    for n in HVDH_FORCED:
        rng = np.random.default_rng([0x4D4, n])
        x = cn(rng, (2, n))
        p = fftj.Plan(T, (n,), kind="c2c", batch=2, opts={"route": 3})
        assert p.route == "HvdhPlan", (n, p.route)
        y = host(p(dev(x, T)))
        tol = 50 * EPS[T]  # runtests.jl:121
        assert rel_l2(y, np.fft.fft(x, axis=-1)) <= tol, (n, rel_l2(y, np.fft.fft(x, axis=-1)) / EPS[T])
        yo = orc.PlanDirect(T, n, "hvdh")(x[0])
        assert rel_l2(y[0], yo) <= tol, (n, rel_l2(y[0], yo) / EPS[T])
        pinv = fftj.Plan(T, (n,), kind="c2c", batch=2, direction=1, scale=1.0 / n, opts={"route": 3})
        xi = host(pinv(dev(y, T)))
        assert rel_l2(xi, x) <= tol, (n, rel_l2(xi, x) / EPS[T])


def test_hvdh_no_coprime_t(fftj):
    """runtests.jl:139: HvdH at n = 390 (an even multiple of 30) has no smooth
    t coprime to n: ArgumentError, as FFTJ._hvdh throws."""
    for T in T_LIST:
        with pytest.raises(fftj.ArgumentError, match="no coprime smooth t"):
            fftj.Plan(T, (390,), kind="c2c", opts={"route": 3})


@pytest.mark.parametrize("T,n,B,route", [(np.float64, 997, 2, 3), (np.float64, 10007, 3, 0), (np.float32, 20011, 2, 0),
                                         (np.float64, 2 * 10007, 2, 0), (np.float32, 13, 2, 3)])
def test_hvdh_factors_fly(fftj, T, n, B, route):
    """FFTJ's factors = :fly (test/runtests.jl:122): the banded solve's
    factors rebuilt on every call (opts.hvdh_factors = 2) agree with the
    tabulated ones (= 1) to rounding, both within 50 eps of FP64 -- by the
    plan's own launches and in a persistent group."""
    import torch
    rng = np.random.default_rng([0xF1F, n])
    x = cn(rng, (B, n))
    pt = fftj.Plan(T, (n,), kind="c2c", batch=B, opts={"route": route, "hvdh_factors": 1})
    pf = fftj.Plan(T, (n,), kind="c2c", batch=B, opts={"route": route, "hvdh_factors": 2})
    assert pf.route == pt.route and pf.route in ("HvdhPlan", "SplitPlan"), pf.route
    xd = dev(x, T)
    yt = host(pt(xd))
    yf = host(pf(xd))
    ref = np.fft.fft(x, axis=-1)
    tol = 50 * EPS[T]  # runtests.jl:121
    assert rel_l2(yt, ref) <= tol and rel_l2(yf, ref) <= tol, (rel_l2(yt, ref) / EPS[T], rel_l2(yf, ref) / EPS[T])
    assert rel_l2(yf, yt) <= 10 * EPS[T], rel_l2(yf, yt) / EPS[T]
    # the same plan as one persistent group (its solve runs the group's copy of the body)
    pg = fftj.Plan(T, (n,), kind="c2c", batch=B, opts={"route": route, "hvdh_factors": 2, "threads_max": 256})
    yg = torch.empty_like(xd)
    g = fftj.Group([pg], [xd], [yg], mode="persistent")
    g()
    g.status()
    assert rel_l2(host(yg), yf) <= 10 * EPS[T], rel_l2(host(yg), yf) / EPS[T]


def _random_nonsmooth(rng, count):
    """Seeded non-smooth lengths n = s p: s 7-smooth in [1, 4096], p a
    product of primes >= 11 (the part no radix covers)."""
    primes = [11, 13, 17, 19, 23, 97, 131, 257, 509, 1009, 2003, 4099]
    out = []
    while len(out) < count:
        s = int(2 ** rng.integers(0, 7) * 3 ** rng.integers(0, 3) * 5 ** rng.integers(0, 2) * 7 ** rng.integers(0, 2))
        p = int(rng.choice(primes))
        if rng.random() < 0.3:
            p *= int(rng.choice(primes[:5]))
        n = s * p
        if 64 <= n <= (1 << 21) and p > 13:
            out.append(n)
    return out


@pytest.mark.parametrize("T", T_LIST)
def test_random_nonsmooth_lengths_all_routes(fftj, T):
    """Seeded random non-smooth lengths on FFTJ's routing and with the route
    forced to resampling (1), Gaussian (2: HvdH / split) and CompositePlan
    (4): forward against FP64 numpy within the parity bar, and the
    normalised inverse round trip."""
    rng = np.random.default_rng(0x5EED if T is np.float32 else 0x5EEE)
    for n in _random_nonsmooth(rng, 10):
        B = 2
        x = cn(rng, (B, n))
        ref = np.fft.fft(x, axis=-1)
        tol = parity_tol(T, n)
        for route in (0, 1, 2, 4):
            pf = fftj.Plan(T, (n,), kind="c2c", batch=B, opts={"route": route})
            y = pf(dev(x, T))
            assert rel_l2(host(y), ref) <= tol, (n, route, pf.route)
            pb = fftj.Plan(T, (n,), kind="c2c", batch=B, direction=1, scale=1.0 / n, opts={"route": route})
            assert rel_l2(host(pb(y)), x) <= 2 * tol, (n, route, pb.route)
