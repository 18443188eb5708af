"""The precision form (plan option precision): radix-16 sub-stages of F32
passes computed as split hi+lo half-precision GEMMs on the tensor cores
(mma.sync m16n8k16, FP32 accumulation, FP32 twiddles), against FP64 numpy on
standard complex normal inputs with 1% of the entries x1e3 (the
dynamic-range stress of the precision-form workload). FP16 hi+lo carries
~22 mantissa bits and must stay within 1e-6 relative L2 and within a small
factor of the plain FP32 form; BF16 hi+lo (~16 bits) within 1e-4."""
import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import fftj
    fftj.build()
    return fftj


def stress(rng, shape):
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)
    flat = x.reshape(-1)
    idx = rng.choice(flat.size, size=max(1, flat.size // 100), replace=False)
    flat[idx] *= 1e3
    return x.astype(np.complex64)


CASES = [((1 << 20,), 2), ((4096,), 8), ((256,), 16), ((1 << 16,), 4), ((4096, 64), 1), ((1 << 12, 1 << 8), 1)]


@pytest.mark.parametrize("dims,batch", CASES)
def test_split_precision_forms(F, dims, batch):
    rng = np.random.default_rng(sum(dims) + batch)
    shape = (batch,) + tuple(reversed(dims)) if batch > 1 else tuple(reversed(dims))
    x = stress(rng, shape)
    axes = tuple(range(-len(dims), 0))
    ref = np.fft.fftn(x.astype(np.complex128), axes=axes)
    xd = torch.from_numpy(x).cuda()
    errs = {}
    for prec in (0, 1, 2):
        p = F.Plan(np.float32, dims, batch=batch, opts={"precision": prec})
        if prec:
            assert p.info.tc_substages >= 1
        y = p(xd)
        torch.cuda.synchronize()
        errs[prec] = rel_l2(y.cpu().numpy(), ref)
    assert errs[0] <= 5e-7, errs
    assert errs[1] <= 1e-6 and errs[1] <= 4 * errs[0] + 1e-7, errs
    assert errs[2] <= 1e-4, errs


def test_split_precision_inverse_round_trip(F):
    rng = np.random.default_rng(7)
    n = 1 << 16
    x = stress(rng, (2, n))
    xd = torch.from_numpy(x).cuda()
    fwd = F.Plan(np.float32, (n,), batch=2, opts={"precision": 1})
    inv = F.Plan(np.float32, (n,), batch=2, direction=1, scale=1.0 / n, opts={"precision": 1})
    back = inv(fwd(xd))
    torch.cuda.synchronize()
    assert rel_l2(back.cpu().numpy(), x) <= 2e-6
