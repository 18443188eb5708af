"""Generates tests/golden/golden.npz: seeded inputs and FP64 reference outputs.

FFTJ's own tests (test/runtests.jl) keep no stored vectors: every testset
draws Xoshiro-seeded randn inputs and compares against FFTW evaluated in
ComplexF64 at run time. Neither Julia nor FFTW exists here, so these fixtures
stand in: the same size lists as the reference testsets (runtests.jl:8,
39-45, 61-63, 114-115, 212, 235-236, 333-335), inputs from numpy's PCG64 with
fixed seeds (FFTJ's Xoshiro streams cannot be reproduced without Julia), and
outputs from numpy's pocketfft in float64 (an independent FFT standing in for
FFTW), cross-checked here against an FP64 direct DFT with compensated sums
(math.fsum) for every length <= 512.

Run: python tests/golden/make_golden.py
"""
import math
import os

import numpy as np

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")

# reference test size lists (test/runtests.jl)
POW2 = [2 ** k for k in range(0, 13)]                                   # :8 (to 2^12 here)
MIXED = [3, 5, 6, 7, 9, 10, 12, 14, 15, 20, 21, 24, 25, 27, 35, 45, 48, 49, 60,
         63, 105, 120, 315, 27 * 32, 3 * 2 ** 8, 9 * 2 ** 8, 5 * 2 ** 8, 7 * 2 ** 8,
         15 * 2 ** 7, 105 * 2 ** 4, 11, 13, 22, 26, 429, 352, 416, 1001,
         11 ** 2 * 2 ** 4, 13 ** 2 * 2 ** 4]                             # :39-45
NONSMOOTH = [17, 19, 23, 34, 38, 51, 97, 101, 289, 331, 361, 997, 1026, 1234, 2050]  # :61-63
HVDH = [11, 13, 17, 19, 22, 23, 26, 34, 38, 46, 97, 101, 202, 331, 997, 1001, 3107, 10007,
        20011]                                                          # :114-115 (65537 at test time)
RAGGED = [3 ** 8, 5 ** 5, 2835, 1000]                                    # :212 subset
REAL = [1, 2, 3, 4, 5, 6, 8, 11, 16, 22, 34, 64, 100, 255, 256, 257, 1024, 768, 1000, 4096]  # :235-236
ND = [(64, 48), (33, 17), (16, 11), (11, 16), (8, 1), (1, 8), (128, 3, 5), (16, 16, 16),
      (12, 10, 14), (32, 64), (60, 50), (24, 40, 3)]                     # :333-335 (FFTJ dims)


def dft_fsum(x, sign=-1):
    n = len(x)
    out = np.empty(n, dtype=np.complex128)
    for k in range(n):
        re, im = [], []
        for j in range(n):
            e = (j * k) % n
            a = 2 * math.pi * e / n
            c, s = math.cos(a), sign * math.sin(a)
            re += [c * x[j].real, -s * x[j].imag]
            im += [c * x[j].imag, s * x[j].real]
        out[k] = complex(math.fsum(re), math.fsum(im))
    return out


def main():
    d = {}
    seed = 0xFF7
    for n in sorted(set(POW2 + MIXED + NONSMOOTH + HVDH + RAGGED)):
        rng = np.random.default_rng([seed, n])
        x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / math.sqrt(2)
        y = np.fft.fft(x)
        if n <= 512:
            ref = dft_fsum(x)
            err = np.linalg.norm(y - ref) / max(np.linalg.norm(ref), 1e-300)
            assert err < 1e-14, (n, err)
        d["c2c_x_%d" % n] = x
        d["c2c_y_%d" % n] = y
    for n in REAL:
        rng = np.random.default_rng([seed + 1, n])
        x = rng.standard_normal(n)
        d["r2c_x_%d" % n] = x
        d["r2c_y_%d" % n] = np.fft.rfft(x)
    for dims in ND:
        key = "x".join(map(str, dims))
        shape = tuple(reversed(dims))  # FFTJ column-major dims -> C-order shape
        rng = np.random.default_rng([seed + 2, len(dims)] + list(dims))
        x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / math.sqrt(2)
        d["nd_x_%s" % key] = x
        d["nd_y_%s" % key] = np.fft.fftn(x)
        xr = rng.standard_normal(shape)
        d["ndr_x_%s" % key] = xr
        d["ndr_y_%s" % key] = np.fft.rfftn(xr)
    # known-answer vectors from the mathematics
    for n in (1, 8, 12, 97, 1024):
        imp = np.zeros(n, dtype=np.complex128)
        imp[0] = 1
        d["kat_impulse_%d" % n] = imp       # -> all ones
        tone = np.exp(2j * np.pi * 3 * np.arange(n) / n) if n > 3 else np.ones(n, dtype=np.complex128)
        d["kat_tone3_%d" % n] = tone        # -> n at bin 3 (n > 3)
    np.savez_compressed(OUT, **d)
    print("wrote", OUT, len(d), "arrays,", os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
