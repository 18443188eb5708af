"""Group executor on the GPU: many plans of mixed dtypes, kinds, lengths and
routes run as one unit -- back-to-back launches, one CUDA graph with parallel
branches, or one persistent work-queue kernel -- and every output matches
numpy's FFT within the parity bar, run after run. Also the persistent
kernel's bounded dependency wait: a wait made to run out (a count nothing
reaches) is reported as FFTJ_ERR_TIMEOUT and the context stays usable."""
import numpy as np
import pytest

from conftest import parity_tol, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# (kind, dtype, n, batch, direction)
ITEMS = [
    ("c2c", np.float32, 4096, 3, -1),
    ("c2c", np.float64, 42525, 2, -1),     # two mixed-radix passes
    ("c2c", np.float32, 1 << 18, 1, -1),   # two passes
    ("c2c", np.float64, 10007, 2, -1),     # HvdH: spread pass, passes, banded solve
    ("c2c", np.float32, 10007, 1, -1),     # resampling: deconvolving pass, interpolation
    ("c2c", np.float64, 64, 5, 1),         # backward, one small pass
    ("r2c", np.float32, 4096, 2, -1),      # even rfft: half-length passes + post-pass
    ("r2c", np.float64, 1009, 1, -1),      # odd rfft: copy, resampled transform, copy
    ("c2r", np.float32, 4096, 2, 1),       # irfft: fused pre-pass load
    ("c2c", np.float32, 1 << 20, 1, -1),   # the largest length of the uneven workload
    ("c2c", np.float64, 3 * 5 * 7 * 11 * 13, 1, -1),
    ("c2c", np.float64, 2 * 10007, 2, -1),  # split route: decimation copy, twiddled banded solve
    ("c2c", np.float64, 16 * 509, 2, -1),   # CompositePlan: s-part passes, twiddled transpose, HvPass lanes
    ("c2c", np.float64, 32 * 131, 2, 1),    # CompositePlan backward with RsPass lanes
    ("c2c", np.float32, 64 * 1031, 1, -1),  # CompositePlan F32 (HvPass)
]


@pytest.fixture(scope="module")
def F():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import fftj
    fftj.build()
    return fftj


def reference(kind, dt, n, b, d, x):
    a = x.cpu().numpy().astype(np.complex128 if kind != "r2c" else np.float64)
    if kind == "c2c":
        return np.fft.fft(a, axis=-1) if d < 0 else np.fft.ifft(a, axis=-1) * n
    if kind == "r2c":
        return np.fft.rfft(a, axis=-1)
    return np.fft.irfft(a, n=n, axis=-1)


def make_case(F, items, seed=11):
    rng = np.random.default_rng(seed)
    plans, xs, ys = [], [], []
    for kind, dt, n, b, d in items:
        p = F.Plan(dt, (n,), kind=kind, direction=d, batch=b, opts={"threads_max": 256})
        shape, tdt = p.in_spec()
        if kind == "c2r":
            h = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
            h[..., 0] = h[..., 0].real
            h[..., -1] = h[..., -1].real
            x = torch.from_numpy(h).to(tdt).cuda()
        elif tdt.is_complex:
            x = torch.from_numpy(rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).to(tdt).cuda()
        else:
            x = torch.from_numpy(rng.standard_normal(shape)).to(tdt).cuda()
        oshape, odt = p.out_spec()
        plans.append(p)
        xs.append(x)
        ys.append(torch.zeros(oshape, dtype=odt, device="cuda"))
    return plans, xs, ys


@pytest.mark.parametrize("mode", ["stream", "graph", "persistent"])
def test_group_matches_numpy_and_repeats(F, mode):
    plans, xs, ys = make_case(F, ITEMS)
    g = F.Group(plans, xs, ys, mode=mode)
    info = g.info
    assert info.nplans == len(ITEMS) and info.nops >= len(ITEMS)
    if mode == "persistent":
        assert info.kernels == 2 and info.ctas >= 1 and info.nitems >= info.nops  # queue reset + queue kernel
    if mode == "graph":
        assert info.branches >= 2
    first = None
    for run in range(2):
        for y in ys:
            y.zero_()
        g()
        g.status()
        torch.cuda.synchronize()
        outs = [y.cpu().numpy().copy() for y in ys]
        for (kind, dt, n, b, d), x, out in zip(ITEMS, xs, outs):
            ref = reference(kind, dt, n, b, d, x)
            err = rel_l2(out, ref)
            assert err <= parity_tol(dt, n), (mode, kind, dt.__name__, n, err)
        if first is None:
            first = outs
        else:  # the same arithmetic on every run, whatever the CTA schedule
            for a, b2 in zip(first, outs):
                assert np.array_equal(a, b2)


def test_persistent_matches_individual_plans(F):
    plans, xs, ys = make_case(F, ITEMS, seed=12)
    g = F.Group(plans, xs, ys, mode="persistent")
    g()
    g.status()
    for p, x, y in zip(plans, xs, ys):
        ref = p(x)
        torch.cuda.synchronize()
        dt = np.float64 if y.dtype in (torch.complex128, torch.float64) else np.float32
        assert rel_l2(y.cpu().numpy(), ref.cpu().numpy()) <= parity_tol(dt, p.n)


def test_group_argument_checks(F):
    plans, xs, ys = make_case(F, ITEMS[:2])
    with pytest.raises(F.ArgumentError):
        F.Group([plans[0], plans[0]], [xs[0], xs[0]], [ys[0], ys[0]])  # a plan twice
    big = F.Plan(np.float32, (8192,), batch=1)  # default F32 plan: 512-thread pass
    xb = torch.zeros(8192, dtype=torch.complex64, device="cuda")
    yb = torch.zeros_like(xb)
    with pytest.raises(F.FFTJError):
        F.Group([big], [xb], [yb], mode="persistent")
    F.Group([big], [xb], [yb], mode="graph")()  # graph and stream modes take any plan
    torch.cuda.synchronize()


def test_persistent_wait_timeout_is_reported(F):
    items = [("c2c", np.float32, 1 << 18, 1, -1), ("c2c", np.float64, 4096, 2, -1)]
    plans, xs, ys = make_case(F, items, seed=13)
    g = F.Group(plans, xs, ys, mode="persistent")
    g.set_wait_limit(2000)  # about a millisecond per wait
    g.debug_stall(1)        # op 1 (the second pass of plan 0) waits for a count never reached
    g()
    with pytest.raises(F.FFTJError, match="gave up"):
        g.status()
    # the context is still usable: a fresh group runs and is correct
    plans2, xs2, ys2 = make_case(F, items, seed=14)
    g2 = F.Group(plans2, xs2, ys2, mode="persistent")
    g2()
    g2.status()
    for (kind, dt, n, b, d), x, y in zip(items, xs2, ys2):
        assert rel_l2(y.cpu().numpy(), reference(kind, dt, n, b, d, x)) <= parity_tol(dt, n)
