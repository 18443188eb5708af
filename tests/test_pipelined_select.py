"""Which passes get the pipelined tensor-copy kernel -- host logic, no GPU.

Dry plans (no tables, no device) run the same selection as real ones and
report it in fftj_plan_info_t.tma_passes: F32 power-of-two passes of a
multi-pass transform whose tile columns are contiguous in HBM (and
three-sub-stage single passes) are pipelined; ComplexF64, odd radices, the
irfft's fused pre-pass, the precision form and plans with opts.plain_loads
keep the one-tile-per-CTA kernels, and so do the last radix-256 passes with
128-byte tile rows (measured faster there)."""
import ctypes

import numpy as np
import pytest

from conftest import ROOT  # noqa: F401  (puts the package on sys.path)


@pytest.fixture(scope="module")
def F():
    import fftj
    fftj.build()
    return fftj


def dry_info(F, kind, dtype, dims, batch=1, **opts):
    from fftj import tune
    q = tune.query(kind, dtype, dims, batch=batch)
    o = F.PlanOpts()
    o.dry = 1
    for k, v in opts.items():
        setattr(o, k, v)
    h = ctypes.c_void_p()
    rc = F.lib().fftj_tune_plan(ctypes.byref(q), ctypes.byref(o), ctypes.byref(h))
    assert rc == 0, F.lib().fftj_last_error_string()
    try:
        info = F.PlanInfo()
        assert F.lib().fftj_plan_get_info(h, ctypes.byref(info)) == 0
        return info
    finally:
        F.lib().fftj_plan_destroy(h)


@pytest.mark.parametrize("kind,dtype,dims,batch,want", [
    ("c2c", np.float32, (1 << 20,), 2, 2),        # 1024 x 1024: both passes
    ("c2c", np.float32, (1 << 18,), 4, 2),        # 512 x 512
    ("c2c", np.float32, (1 << 26,), 1, 2),        # 512 x 512 x 256: the last radix-256 pass keeps plain loads
    ("c2c", np.float32, (4096, 4096), 1, 3),      # radix-4096 row pass + two radix-64 column passes
    ("c2c", np.float32, (4096,), 5, 1),           # three-sub-stage single pass
    ("c2c", np.float32, (256,), 8, 0),            # two-sub-stage single pass
    ("c2c", np.float32, (42525,), 2, 0),          # odd radices
    ("c2c", np.float64, (1 << 18,), 4, 0),        # ComplexF64 (fixed point, ALU bound)
    ("r2c", np.float32, (1 << 25,), 4, 2),        # half-length passes; the last one keeps plain loads
    ("c2r", np.float32, (1 << 25,), 4, 1),        # the first pass carries the fused pre-pass
])
def test_pipelined_pass_selection(F, kind, dtype, dims, batch, want):
    info = dry_info(F, kind, dtype, dims, batch=batch)
    assert info.tma_passes == want, (kind, dims, list(info.pass_radix[:info.npasses]))


def test_options_turn_the_pipeline_off(F):
    assert dry_info(F, "c2c", np.float32, (1 << 20,), 2).tma_passes == 2
    assert dry_info(F, "c2c", np.float32, (1 << 20,), 2, plain_loads=1).tma_passes == 0
    # the FP16 precision form runs in the pipelined kernels' tensor-core
    # variants (first sub-stage radix 16 on tcgen05); BF16 and plain_loads
    # keep the run-time-radix kernel
    fp16 = dry_info(F, "c2c", np.float32, (1 << 20,), 2, precision=1)
    assert fp16.tma_passes == 2 and fp16.tc_substages == 2
    assert dry_info(F, "c2c", np.float32, (1 << 20,), 2, precision=2).tma_passes == 0
    assert dry_info(F, "c2c", np.float32, (1 << 20,), 2, precision=1, plain_loads=1).tma_passes == 0
    # passes without a radix-16 first sub-stage keep the plain pipelined kernel
    rows = dry_info(F, "c2c", np.float32, (4096, 4096), 1, precision=1)
    assert rows.tma_passes == 3 and rows.tc_substages == 1


def test_schedule_hash_tells_the_kernels_apart(F):
    a = dry_info(F, "c2c", np.float32, (1 << 20,), 2)
    b = dry_info(F, "c2c", np.float32, (1 << 20,), 2, plain_loads=1)
    assert a.schedule_hash != b.schedule_hash
    assert list(a.pass_radix[:a.npasses]) == list(b.pass_radix[:b.npasses])
