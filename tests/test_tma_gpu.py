"""Pipelined tensor-copy passes on the GPU.

F32 power-of-two passes of multi-pass transforms run as persistent,
double-buffered kernels whose tiles arrive by TMA tensor copies. They do the
same arithmetic as the one-tile-per-CTA kernels, so:
- every case matches numpy's FFT within the parity bar and is bit-identical
  to the same plan built with plain loads (opts plain_loads = 1);
- an input that is not 16-byte aligned (no tensor map) runs the plain kernel
  for that pass and gives the same bits;
- the bounded wait: tile barriers made to expect bytes that never arrive
  (debug_stall) run out, the plan reports FFTJ_ERR_TIMEOUT, and the context
  stays usable (the next execution is correct).
"""
import numpy as np
import pytest

from conftest import parity_tol, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import fftj
    fftj.build()
    return fftj


# (kind, dims (column-major), batch, direction)
CASES = [
    ("c2c", (1 << 20,), 2, -1),       # 1024 x 1024: radix 16*8*8, 8 columns per tile
    ("c2c", (1 << 18,), 4, -1),       # 512 x 512: radix 8*8*8
    ("c2c", (1 << 18,), 2, 1),        # backward
    ("c2c", (1 << 16,), 8, -1),       # 256 x 256: radix 16*16, 16 columns
    ("c2c", (1 << 12, 1 << 12), 1, -1),  # 2-D: the strided axis as two radix-64 passes
    ("c2c", (1024, 1024), 2, 1),      # 2-D: strided radix-1024 pass
    ("r2c", (1 << 21,), 2, -1),       # rfft: half-length passes + post-pass
    ("c2c", (4096,), 5, -1),          # single pass, radix 16*16*16, one transform per tile
    ("c2c", (2048,), 37, -1),         # single pass, two per tile: the last tile holds one
    ("c2c", (1024,), 13, 1),          # single pass, four per tile, backward
    ("c2c", (512,), 9, -1),           # single pass, radix 8*8*8, eight per tile
]


def make_input(shape, tdt, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    if tdt.is_complex:
        rdt = torch.float32
        return torch.complex(torch.randn(shape, generator=g, device="cuda", dtype=rdt),
                             torch.randn(shape, generator=g, device="cuda", dtype=rdt))
    return torch.randn(shape, generator=g, device="cuda", dtype=tdt)


def reference(kind, dims, d, x):
    a = x.cpu().numpy().astype(np.complex128 if kind == "c2c" else np.float64)
    axes = tuple(range(a.ndim - len(dims), a.ndim))
    if kind == "r2c":
        return np.fft.rfftn(a, axes=axes[::-1])
    return np.fft.fftn(a, axes=axes) if d < 0 else np.fft.ifftn(a, axes=axes) * np.prod(dims)


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s_%s_b%d_d%d" % (c[0], "x".join(map(str, c[1])), c[2], c[3]))
def test_pipelined_passes_match_numpy_and_plain_loads(F, case):
    kind, dims, batch, d = case
    p = F.Plan(np.float32, dims, kind=kind, batch=batch, direction=d)
    q = F.Plan(np.float32, dims, kind=kind, batch=batch, direction=d, opts={"plain_loads": 1})
    assert p.info.tma_passes >= 1, "expected pipelined passes"
    assert q.info.tma_passes == 0
    shape, tdt = p.in_spec()
    x = make_input(shape, tdt, 7)
    y = p(x)
    p.status()
    y2 = q(x)
    torch.cuda.synchronize()
    assert torch.equal(y, y2), "pipelined and plain-load kernels must give the same bits"
    n = int(np.prod(dims))
    err = rel_l2(y.cpu().numpy(), reference(kind, dims, d, x))
    assert err <= parity_tol(np.float32, n), err


def test_unaligned_input_runs_the_plain_kernel(F):
    n, batch = 1 << 18, 2
    p = F.Plan(np.float32, (n,), batch=batch)
    base = make_input((n * batch + 1,), torch.complex64, 9)
    x = base[1:].view(batch, n)  # 8-byte offset: no tensor map for the first pass
    assert x.data_ptr() % 16 == 8
    y = p(x)
    p.status()
    y_ref = p(x.clone())  # aligned copy: pipelined first pass
    torch.cuda.synchronize()
    assert torch.equal(y, y_ref)
    assert rel_l2(y.cpu().numpy(), np.fft.fft(x.cpu().numpy().astype(np.complex128), axis=-1)) <= parity_tol(np.float32, n)


def test_wait_timeout_is_reported(F):
    n, batch = 1 << 18, 2
    p = F.Plan(np.float32, (n,), batch=batch)
    assert p.info.tma_passes >= 1
    x = make_input((batch, n), torch.complex64, 11)
    p.set_wait_limit(1_000_000)  # 1 ms per wait
    p.debug_stall(16)            # every tile barrier waits for 16 bytes that never arrive
    p(x)
    with pytest.raises(F.FFTJError, match="gave up"):
        p.status()
    # the context is still usable and the status was cleared
    p.debug_stall(0)
    p.set_wait_limit(1_000_000_000)
    y = p(x)
    p.status()
    err = rel_l2(y.cpu().numpy(), np.fft.fft(x.cpu().numpy().astype(np.complex128), axis=-1))
    assert err <= parity_tol(np.float32, n), err


def test_pipelined_equals_plain_on_random_shapes(F):
    """Seeded random power-of-two shapes, batches, directions and kinds: the
    plan with pipelined passes and the plain-load plan give the same bits."""
    rng = np.random.default_rng(2024)
    checked = 0
    for _ in range(40):
        kind = rng.choice(["c2c", "c2c", "r2c", "c2r"])
        rank = int(rng.choice([1, 1, 2, 3]))
        if rank == 1:
            dims = (1 << int(rng.integers(9, 22)),)
        elif rank == 2:
            dims = tuple(1 << int(v) for v in rng.integers(5, 12, size=2))
        else:
            dims = tuple(1 << int(v) for v in rng.integers(4, 8, size=3))
        total = int(np.prod(dims))
        batch = int(rng.integers(1, 6)) if total <= (1 << 20) else 1
        d = -1 if kind == "r2c" else (1 if kind == "c2r" else int(rng.choice([-1, 1])))
        seed = int(rng.integers(1 << 30))
        p = F.Plan(np.float32, dims, kind=kind, batch=batch, direction=d)
        if p.info.tma_passes == 0:
            continue
        q = F.Plan(np.float32, dims, kind=kind, batch=batch, direction=d, opts={"plain_loads": 1})
        shape, tdt = p.in_spec()
        x = make_input(shape, tdt, seed)
        if kind == "c2r":  # a spectrum of real data: DC and Nyquist bins real
            x[..., 0].imag.zero_()
            x[..., -1].imag.zero_()
        y = p(x)
        p.status()
        y2 = q(x)
        torch.cuda.synchronize()
        assert torch.equal(y, y2), (kind, dims, batch, d)
        checked += 1
    assert checked >= 15, checked
