"""Generates bfly_consts.h: cos/sin(2*pi*j*k/P) for the odd-prime butterflies
(P = 3, 5, 7, 11, 13; j, k = 1..(P-1)/2), the conjugate-pair DFT that FFTJ's
bfp uses (src/kernels.jl:146-228). Values are correctly rounded doubles from
mpmath when available, else from math.cos/sin of an exactly reduced angle."""
import math
import os

try:
    import mpmath as mp
    mp.mp.prec = 200
    def cs(num, den):
        a = 2 * mp.pi * num / den
        return float(mp.cos(a)), float(mp.sin(a))
except ImportError:  # pragma: no cover
    def cs(num, den):
        a = 2 * math.pi * num / den
        return math.cos(a), math.sin(a)

def fn(name, vals):
    # a constexpr lookup usable from host and device code; with a constant
    # index (unrolled loops) it folds to an immediate
    body = " : ".join("i == %d ? %r" % (i, v) for i, v in enumerate(vals[:-1]))
    body = (body + " : " if body else "") + repr(vals[-1])
    return "__host__ __device__ constexpr double %s(int i) { return %s; }" % (name, body)


lines = ["// Generated by gen_bfly_consts.py -- do not edit.", "#pragma once", "#include <cuda_runtime.h>", "namespace fftj {"]
for P in (3, 5, 7, 11, 13):
    h = (P - 1) // 2
    cc, ss = [], []
    for k in range(1, h + 1):
        for j in range(1, h + 1):
            c, s = cs((j * k) % P, P)
            cc.append(c)
            ss.append(s)
    lines.append(fn("kCos%d" % P, cc))
    lines.append(fn("kSin%d" % P, ss))
c16 = [cs(t, 16) for t in range(16)]
lines.append(fn("kCos16", [c for c, _ in c16]))
lines.append(fn("kSin16", [s for _, s in c16]))
lines.append("}  // namespace fftj")
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bfly_consts.h")
with open(out, "w") as f:
    f.write("\n".join(lines) + "\n")
