"""The oracle (CPU restatement of FFTJ.jl) pinned against the golden vectors,
an FP64 direct DFT and the reference test suite's identities and routing.
CPU only."""
import numpy as np
import pytest

from conftest import EPS, rel_l2

# tolerance classes of test/runtests.jl: 50 eps (smooth, four-step), 100 eps
# (resampling, real), 200 eps (N-d)
T_LIST = [np.float32, np.float64]


def _golden_sizes(golden, prefix):
    return sorted(int(k[len(prefix):]) for k in golden.files if k.startswith(prefix))


@pytest.mark.parametrize("T", T_LIST)
def test_c2c_matches_golden(golden, orc, T):
    for n in _golden_sizes(golden, "c2c_x_"):
        x = golden["c2c_x_%d" % n]
        ref = golden["c2c_y_%d" % n]
        p = orc.Plan1D(T, n, "fft")
        y = p(x)
        k = 100 if p.route == "ResamplePlan" else 50
        assert rel_l2(y, ref) <= k * EPS[T], (n, p.route, rel_l2(y, ref) / EPS[T])
        # round trip (runtests.jl:23) and bfft = n * ifft (runtests.jl:76)
        xi = orc.Plan1D(T, n, "ifft")(y)
        assert rel_l2(xi, x) <= 2 * k * EPS[T], n
        xb = orc.Plan1D(T, n, "bfft")(ref.astype(np.complex128))
        assert rel_l2(xb, n * x) <= 2 * k * EPS[T], n


def test_direct_dft_matches_golden(golden, orc):
    for n in _golden_sizes(golden, "c2c_x_"):
        if n > 1100:
            continue
        x = golden["c2c_x_%d" % n]
        assert rel_l2(orc.dft_f64(x), golden["c2c_y_%d" % n]) <= 4 * EPS[np.float64], n


def test_known_answers(golden, orc):
    for key in golden.files:
        if not key.startswith("kat_"):
            continue
        n = int(key.rsplit("_", 1)[1])
        x = golden[key]
        for T in T_LIST:
            y = orc.Plan1D(T, n, "fft")(x)
            if "impulse" in key:
                assert np.allclose(y, np.ones(n), atol=10 * EPS[T])
            elif n > 3:
                exp = np.zeros(n, dtype=np.complex128)
                exp[3] = n
                assert rel_l2(y, exp) <= 50 * EPS[T] * max(np.log2(n), 1), key


@pytest.mark.parametrize("T", T_LIST)
def test_rfft_matches_golden(golden, orc, T):
    for n in _golden_sizes(golden, "r2c_x_"):
        x = golden["r2c_x_%d" % n]
        ref = golden["r2c_y_%d" % n]
        y = orc.PlanReal(T, n, "rfft")(x)
        assert y.shape == (n // 2 + 1,)
        assert rel_l2(y, ref) <= 100 * EPS[T], n
        xr = orc.PlanReal(T, n, "irfft")(ref)
        assert rel_l2(xr, x) <= 100 * EPS[T], n
        xb = orc.PlanReal(T, n, "brfft")(ref)
        assert rel_l2(xb, n * x) <= 100 * EPS[T], n


@pytest.mark.parametrize("T", T_LIST)
def test_nd_matches_golden(golden, orc, T):
    for key in golden.files:
        if not key.startswith("nd_x_"):
            continue
        dims = [int(v) for v in key[5:].split("x")]
        x = golden[key]
        ref = golden["nd_y_" + key[5:]]
        y = orc.PlanND(T, dims, "fft")(x)
        assert rel_l2(y, ref) <= 200 * EPS[T], dims
        assert rel_l2(orc.PlanND(T, dims, "ifft")(ref), x) <= 200 * EPS[T], dims
        xr = golden["ndr_x_" + key[5:]]
        rref = golden["ndr_y_" + key[5:]]
        Y = orc.PlanND(T, dims, "rfft")(xr)
        assert Y.shape == rref.shape and rel_l2(Y, rref) <= 200 * EPS[T], dims
        assert rel_l2(orc.PlanND(T, dims, "irfft")(rref), xr) <= 200 * EPS[T], dims
        assert rel_l2(orc.PlanND(T, dims, "brfft")(rref), np.prod(dims) * xr) <= 200 * EPS[T], dims


def test_routing_matches_reference_table(orc):
    """Plan types asserted by the reference's routing tests
    (test/runtests.jl:391-419). Those assertions hold for a 512-bit (AVX-512)
    host only (e.g. F32 40000 threaded is four-step only when W = 16), so the
    oracle is pinned at 512 bits here; the config splits below hold on the
    128-bit NEON host of the GPU machine as well."""
    orc.set_vector_bits(512)
    r = lambda T, n, nt=1: orc.Plan1D(T, n, "fft", nthreads=nt).route
    for n in (405, 11 * 1024, 4000):
        assert r(np.float64, n) == "FFTPlan"
    assert r(np.float32, 8000) == "FFTPlan"
    for n in (2835, 3 ** 8, 2 * 3 ** 6 * 5 ** 2 * 7 ** 2, 13 ** 3):
        assert r(np.float64, n) == "FourStepPlan", n
    assert r(np.float64, 12000) == "FFTPlan"
    assert r(np.float32, 40000) == "FFTPlan"
    assert r(np.float32, 40000, 4) == "FourStepPlan"
    assert r(np.float64, 2 ** 17) == "FFTPlan"
    assert r(np.float64, 2 ** 18) == "FourStepPlan"
    assert r(np.float64, 2 ** 15, 4) == "FourStepPlan"
    assert r(np.float64, 2 ** 14, 4) == "FFTPlan"
    assert r(np.float64, 10006) == "ResamplePlan"
    assert r(np.float32, 10007) == "ResamplePlan"
    assert r(np.float32, 729) == "ResamplePlan"
    assert r(np.float32, 2187) == "FourStepPlan"
    assert r(np.float32, 3 ** 12) == "FourStepPlan"
    # the config sizes (four-step splits of the reference's planner)
    orc.set_vector_bits(128)
    assert orc.Plan1D(np.float32, 42525, "fft").info()[2:4] == [225, 189]
    assert orc.Plan1D(np.float64, 2 ** 18, "fft").info()[2:4] == [512, 512]
    m, w, _ = orc.resample_params(np.float32, 10007)
    assert (m, w) == (20480, 8)
    m, w, _ = orc.resample_params(np.float64, 10007)
    assert (m, w) == (20480, 16)
    orc.set_vector_bits(512)
    assert orc.Plan1D(np.float32, 42525, "fft").info()[2:4] == [225, 189]
    orc.set_vector_bits(128)


@pytest.mark.parametrize("T", T_LIST)
def test_threaded_bitwise_serial(orc, T):
    """test/threading.jl: threaded plans are bitwise equal to serial ones of
    the same algorithm (deterministic tforeach chunking)."""
    rng = np.random.default_rng(5)
    for n in (2 ** 17, 3 * 2 ** 16, 42525):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        p4 = orc.Plan1D(T, n, "fft", nthreads=4)
        info = p4.info()
        y4 = p4(x)
        if p4.route == "FourStepPlan":
            # same split, one task: the serial plan of FFTJ's _serial_copy
            y1 = orc.Plan1D(T, n, "fft", nthreads=1)(x)
            if orc.Plan1D(T, n, "fft", nthreads=1).info()[2:4] == info[2:4]:
                assert np.array_equal(y1, y4), n
        assert rel_l2(y4, np.fft.fft(x)) <= 50 * EPS[T]


# ---------------------------------------------------------------------------
# Gaussian resampling (HvdhPlan), CompositePlan and SplitPlan restatements,
# at the reference's own test sizes and tolerance classes.

# test/runtests.jl:114-115
HVDH_SIZES = [11, 13, 17, 19, 22, 23, 26, 34, 38, 46, 97, 101, 202, 331, 997, 1001, 3107, 10007,
              20011, 65537]
# test/runtests.jl:148-150 (filtered by _use_composite per dtype)
COMPOSITE_SIZES = [17 * 1024, 101 * 64, 1009 * 16, 19 * 3072, 17 * 2 ** 13, 101 * 1024, 1009 * 64,
                   10007 * 32, 17 * 19 * 512, 3 ** 4 * 5 * 7 * 101]
# test/runtests.jl:88-89
SPLIT_SIZES = [2 * 1009, 6 * 1009, 14 * 1009, 2 * 10007, 4 * 10007, 12 * 2003, 2 * 32771, 8 * 16411,
               2 * 65537]


def _smooth_part(n):  # src/composite.jl:43-51
    s = 1
    for f in (2, 3, 5, 7):
        while n % (s * f) == 0:
            s *= f
    return s


def _use_hvdh(T, n):  # src/hvdh.jl:97
    return n % 2 == 1 and n >= (1000 if T == np.float64 else 16384)


def _use_composite(T, n):  # src/composite.jl:53-54
    return n >= (4096 if T == np.float64 else 32768) and _smooth_part(n) >= 16


def _use_split(T, n):  # src/composite.jl:131-135
    s = _smooth_part(n)
    return n % 2 == 0 and s < 16 and _use_hvdh(T, n // s) and n >= (16384 if T == np.float64 else 65536)


def _smooth13(n):
    for p in (2, 3, 5, 7, 11, 13):
        while n % p == 0:
            n //= p
    return n == 1


def _input(golden, n, seed):
    key = "c2c_x_%d" % n
    if key in golden.files:
        return golden[key], golden["c2c_y_%d" % n]
    rng = np.random.default_rng([seed, n])
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)
    return x, np.fft.fft(x)


@pytest.mark.parametrize("T", T_LIST)
def test_hvdh_reference_sizes(golden, orc, T):
    """runtests.jl:110-137: FFTJ._hvdh at every size within 50 eps of FFTW
    (here: the golden FP64 outputs / numpy), :fly factors equal to the
    tabulated ones, the inverse round trip within 50 eps, and plan_fft's route
    for non-smooth lengths."""
    ct = np.complex64 if T == np.float32 else np.complex128
    for n in HVDH_SIZES:
        x, ref = _input(golden, n, 0x4D4)
        x = x.astype(ct)
        p = orc.PlanDirect(T, n, "hvdh", factors="table")
        y = p(x)
        assert rel_l2(y, ref) <= 50 * EPS[T], (n, rel_l2(y, ref) / EPS[T])
        yf = orc.PlanDirect(T, n, "hvdh", factors="fly")(x)
        assert np.array_equal(y, yf), n
        pinv = orc.PlanDirect(T, n, "hvdh", direction="ifft")
        assert rel_l2(pinv(y), x) <= 50 * EPS[T], n
        if not _smooth13(n):
            route = orc.Plan1D(T, n, "fft").route
            if _use_hvdh(T, n) and not _use_composite(T, n):
                assert route == "HvdhPlan", (n, route)
            else:
                assert route in ("ResamplePlan", "CompositePlan", "SplitPlan"), (n, route)


def test_hvdh_no_coprime_t():
    """runtests.jl:139: even multiples of 30 have no coprime smooth t."""
    from oracle import oracle as O
    for T in T_LIST:
        with pytest.raises(ValueError, match="no coprime smooth t"):
            O.PlanDirect(T, 390, "hvdh")


def test_hvdh_bfft_20011(orc):
    """runtests.jl:140-143: plan_bfft routes 20011 to HvdH, and bfft(fft(x))
    = n x within 50 eps."""
    for T in T_LIST:
        ct = np.complex64 if T == np.float32 else np.complex128
        rng = np.random.default_rng(0x4D4)
        x = (rng.standard_normal(20011) + 1j * rng.standard_normal(20011)).astype(ct)
        pb = orc.Plan1D(T, 20011, "bfft")
        assert pb.route == "HvdhPlan"
        assert rel_l2(pb(orc.Plan1D(T, 20011, "fft")(x)), 20011 * x.astype(np.complex128)) <= 50 * EPS[T]


@pytest.mark.parametrize("T", T_LIST)
def test_composite_reference_sizes(orc, T):
    """runtests.jl:146-170: plan_fft routes these to CompositePlan; within
    100 eps of FFTW; ifft round trip and bfft = n x."""
    ct = np.complex64 if T == np.float32 else np.complex128
    ns = [n for n in COMPOSITE_SIZES if _use_composite(T, n)]
    assert len(ns) >= 4
    for n in ns:
        rng = np.random.default_rng([0xC0B, n])
        x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(ct)
        ref = np.fft.fft(x.astype(np.complex128))
        p = orc.Plan1D(T, n, "fft")
        assert p.route == "CompositePlan", (n, p.route)
        y = p(x)
        assert rel_l2(y, ref) <= 100 * EPS[T], (n, rel_l2(y, ref) / EPS[T])
        assert rel_l2(orc.Plan1D(T, n, "ifft")(y), x) <= 100 * EPS[T], n
        assert rel_l2(orc.Plan1D(T, n, "bfft")(y), n * x.astype(np.complex128)) <= 100 * EPS[T], n


@pytest.mark.parametrize("T", T_LIST)
def test_split_reference_sizes(orc, T):
    """runtests.jl:84-107: FFTJ._split within 100 eps of FFTW; plan_fft takes
    SplitPlan where _use_split holds; the inverse round trip."""
    ct = np.complex64 if T == np.float32 else np.complex128
    for n in SPLIT_SIZES:
        rng = np.random.default_rng([0x5B1, n])
        x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(ct)
        ref = np.fft.fft(x.astype(np.complex128))
        y = orc.PlanDirect(T, n, "split")(x)
        assert rel_l2(y, ref) <= 100 * EPS[T], (n, rel_l2(y, ref) / EPS[T])
        if _use_split(T, n):
            assert orc.Plan1D(T, n, "fft").route == "SplitPlan", n
        assert rel_l2(orc.PlanDirect(T, n, "split", direction="ifft")(y), x) <= 100 * EPS[T], n


def test_fs2_routing_and_parity(orc):
    """FFTJ's _ndplan runs a 2-D complex plan through Fs2Plan (the strided
    dim 2 in strips, then the rows) when _use_fs2 holds (src/fourstep.jl:
    518-529: >= 4 MB serially, strip and inner-buffer limits, a fused
    power-of-two last row stage); the restated plan routes the same way and
    matches FP64 numpy within the parity bar."""
    from conftest import parity_tol, rel_l2
    assert orc.PlanND(np.float32, [4096, 4096], "fft").route == "Fs2Plan"
    assert orc.PlanND(np.float64, [1024, 1024], "fft").route == "Fs2Plan"
    assert orc.PlanND(np.float32, [512, 512], "fft").route == "NdPlan"    # 2 MB: below the serial 4 MB
    assert orc.PlanND(np.float32, [64, 4096], "fft").route == "NdPlan"    # strips too wide for the inner buffer
    assert orc.PlanND(np.float32, [16, 16, 4], "fft").route == "NdPlan"   # 3-D
    rng = np.random.default_rng(0xF52)
    for T, shape in ((np.float64, (1024, 1024)), (np.float32, (1024, 2048))):
        x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        p = orc.PlanND(T, list(reversed(shape)), "fft")
        assert p.route == "Fs2Plan"
        y = p(x)
        ref = np.fft.fft2(x)
        assert rel_l2(y, ref) <= parity_tol(T, x.size), (T, shape)
        xi = orc.PlanND(T, list(reversed(shape)), "ifft")(y)
        assert rel_l2(xi, x) <= 2 * parity_tol(T, x.size)


def test_batched_dim1_edges(orc):
    """FFTJ's N-d plans run the dim-1 edge batched, pencils as vector lanes,
    on a chain built without the small-stride layout: the complex dim-1 pass
    when its per-pencil chain would not get the fused edge and the pencils
    fill the lanes (src/ndplan.jl:72-77), and the real edge under
    _real_batched (src/ndplan.jl:343-353), whose inverse folds every
    normalization into the pre-pass factor (:466-469). The restated plans
    choose the same way and match FP64 numpy within the parity bar."""
    from conftest import parity_tol, rel_l2
    # 128-bit host (4 F32 / 2 F64 lanes)
    assert not orc.PlanND(np.float32, [64, 8], "rfft").batched       # h = 32: fused 4·8 pencil
    assert orc.PlanND(np.float32, [48, 3, 3], "rfft").batched        # h = 24: 3·8, no fused edge
    assert not orc.PlanND(np.float32, [48, 3, 3], "fft").batched     # 4·3·4: fused edge
    assert orc.PlanND(np.float32, [12, 10], "fft").batched           # 4·3: one stride-1 radix 4 too short
    assert not orc.PlanND(np.float32, [14, 2], "irfft").batched      # 2 pencils < 4 lanes
    assert not orc.PlanND(np.float32, [256, 256, 256], "rfft").batched  # the 256^3 rfft: fused pencils
    try:
        orc.set_vector_bits(512)                                     # 16 F32 lanes
        assert orc.PlanND(np.float32, [64, 32], "rfft").batched      # h = 32: no small first stage at W = 16
        assert orc.PlanND(np.float32, [128, 16], "rfft").batched     # fused, but 65 x 16 x 4 B is L2-resident
        assert not orc.PlanND(np.float32, [128, 2048], "rfft").batched  # fused and 532 KB > 512 KB
    finally:
        orc.set_vector_bits(128)
    rng = np.random.default_rng(0xBA7)
    for T in (np.float32, np.float64):
        for dims in ([48, 3, 3], [40, 4], [12, 10], [2, 16], [1536, 8]):
            shape = tuple(reversed(dims))
            x = rng.standard_normal(shape)
            n = x.size
            Y = orc.PlanND(T, dims, "rfft")(x)
            ref = np.fft.rfftn(x)
            assert rel_l2(Y, ref) <= parity_tol(T, n), (T, dims)
            assert rel_l2(orc.PlanND(T, dims, "irfft")(ref), x) <= parity_tol(T, n), (T, dims)
            assert rel_l2(orc.PlanND(T, dims, "brfft")(ref), n * x) <= parity_tol(T, n), (T, dims)
            xc = x + 1j * rng.standard_normal(shape)
            assert rel_l2(orc.PlanND(T, dims, "fft")(xc), np.fft.fftn(xc)) <= parity_tol(T, n), (T, dims)


def test_vexp_and_hvdh_recurrences(orc):
    """FFTJ's HvdH seeds its Gaussian recurrences with its own polynomial exp
    (_vexp, src/hvdh.jl:99-114: Cody-Waite reduction, 14 / 8 Taylor terms):
    the restated one stays within 2 ulp of the correctly rounded exp over the
    arguments the seeds see, and the restated HvdH (band columns re-seeded
    every 4, spread states every 8 vectors) stays within FFTJ's 50 eps."""
    from conftest import rel_l2
    from oracle import oracle as O
    import math
    for T in T_LIST:
        xs = np.linspace(-10.0, 10.0, 2001).astype(T)
        for x in xs:
            e = O.vexp(T, float(x))
            ref = math.exp(float(x))
            ulp = float(np.spacing(T(ref)))
            assert abs(e - ref) <= 2 * ulp, (T, float(x), e, ref)
    rng = np.random.default_rng(0xE1)
    for T in T_LIST:
        ct = np.complex64 if T == np.float32 else np.complex128
        for n in (1001, 16385, 65537):
            x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(ct)
            y = orc.PlanDirect(T, n, "hvdh")(x)
            assert rel_l2(y, np.fft.fft(x.astype(np.complex128))) <= 50 * EPS[T], (T, n)


def test_resample_polynomial_weights(orc):
    """A 1-D ResamplePlan whose weight table would exceed _RS_TABLE_MAX
    (2 MiB: n w sizeof(T)) evaluates Chebyshev-fitted piecewise polynomials
    instead (src/resample.jl:123-169, 229-250): Float32 8 x 10007 = 80056
    (w = 8, 2.6 MB) routes to ResamplePlan with polynomial weights, 60002 (1.9
    MB) keeps the table; both within FFTJ's 50 eps of FP64."""
    from conftest import rel_l2
    rng = np.random.default_rng(0x9017)
    for n, poly in ((80056, True), (60002, False)):
        p = orc.Plan1D(np.float32, n, "fft")
        route, n_, m, w, deg = p.info()[:5]
        assert p.route == "ResamplePlan" and w == 8 and (deg > 0) == poly, (n, p.info())
        x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
        ref = np.fft.fft(x.astype(np.complex128))
        assert rel_l2(p(x), ref) <= 50 * EPS[np.float32], n
        assert rel_l2(orc.Plan1D(np.float32, n, "ifft")(ref), x) <= 50 * EPS[np.float32], n
