// Block fixed-point arithmetic of the ComplexF64 passes.
//
// GB300 runs FP64 at 1/64 of the FP32 rate (1.19 TFLOP/s measured with an
// FMA loop), so a ComplexF64 Stockham pass done in FP64 is bound by the FP64
// pipe at 7-10% of the HBM bandwidth. The passes here keep the data FP64 in
// HBM but compute each tile column in 64-bit fixed point on the integer
// pipes: when a column of R points arrives, its largest exponent E is found
// and every point becomes round(x * 2^K), K = B + 1022 - E, so that every
// component is below 2^B, B = 61 - ceil(log2 r0) for the pass's first
// sub-stage radix r0 (an input within B - 53 binades of the column's largest
// is represented exactly). Bound on complex magnitudes: a radix-r sub-stage
// takes magnitudes below A to below r A (every partial sum, the radix-8
// butterfly's (re + im) sums and the odd-prime banks included; twiddles keep
// magnitudes), so with A < 2^62 / r before each sub-stage no value reaches
// 2^62; each sub-stage's outputs are shifted right by ceil(log2 r') for the
// next radix r' to restore that, and the final scale is 2^(K - shifts). Sums
// and differences are exact int64 additions; the products by twiddles and
// DFT constants and the shifts round by about one unit, which is tiny next
// to the grown values. Constants and twiddles are Q61: round(c * 2^61),
// |c| <= 1, clamped to 2^61 - 1. A product c * x splits both operands at bit 31
// (c = ch 2^31 + cl, x = xh 2^31 + xl, cl, xl in [0, 2^31)):
//   c x / 2^61 = 2 ch xh + (ch xl + cl xh) / 2^30 + cl xl / 2^61,
// kept as three 32x32->64 multiply-adds and a shift; the multiply-add chain
// starts from 2^30, which rounds the shift to nearest and adds the mean
// (half a unit) of the dropped last term.
//
// Conversions use integer instructions only: on GB300 an int64 -> double
// conversion issues two FP64-pipe instructions, and FP64 work that the
// compiler predicates (rather than branches around) is issued for every
// element, so the rare cases (results outside the normal double range) sit
// in a separate non-inlined function.
//
// Precision: inputs are exact unless they are more than B - 53 binades
// below their column's largest (then rounded to half a unit of 2^-K); the
// output is rounded to nearest (ties to even) into a double, so a pass's
// error is close to one double rounding, below an FP64 pass's. Columns
// holding an Inf or NaN produce NaN outputs.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace fftj {

__host__ __device__ constexpr long long fx_q61(double c) {
  // round(c * 2^61) clamped to [-2^61, 2^61 - 1] (|c| <= 1)
  return c >= 1.0 ? (1ll << 61) - 1
                  : c <= -1.0 ? -(1ll << 61)
                              : (long long)(c * 2305843009213693952.0 + (c >= 0 ? 0.5 : -0.5));
}

struct Fx {
  long long v;
  Fx() = default;
  // a Q61 constant (DFT constants, 1, 0)
  __host__ __device__ constexpr Fx(double c) : v(fx_q61(c)) {}
  __host__ __device__ constexpr Fx(int c) : v(fx_q61((double)c)) {}
  __host__ __device__ static constexpr Fx raw(long long x) {
    Fx f(0);
    f.v = x;
    return f;
  }
  // Arithmetic as hidden friends: found only for Fx arguments, so the
  // float/double fma and operators of the same code stay the built-in ones.
  friend __device__ __forceinline__ Fx operator+(Fx a, Fx b) { return raw(a.v + b.v); }
  friend __device__ __forceinline__ Fx operator-(Fx a, Fx b) { return raw(a.v - b.v); }
  friend __device__ __forceinline__ Fx operator-(Fx a) { return raw(-a.v); }
  // c * x / 2^61: c a Q61 constant or twiddle (first operand), x a value
  // (|x| < 2^62)
  friend __device__ __forceinline__ Fx operator*(Fx c, Fx x) {
    const int ch = (int)(c.v >> 31), cl = (int)(c.v & 0x7fffffff);
    const int xh = (int)(x.v >> 31), xl = (int)(x.v & 0x7fffffff);
    const long long mid = (long long)ch * xl + ((long long)cl * xh + (1ll << 30));
    return raw((long long)(2 * ch) * xh + (mid >> 30));
  }
  friend __device__ __forceinline__ Fx fma(Fx c, Fx x, Fx a) { return c * x + a; }
};

struct alignas(16) Fx2 {
  Fx x, y;
};

// a product of two Q61 twiddles brought back into the Q61 range
__device__ __forceinline__ Fx fx_clamp_q61(Fx w) {
  constexpr long long top = (1ll << 61) - 1;
  return Fx::raw(w.v > top ? top : (w.v < -top ? -top : w.v));
}

// ---------------------------------------------------------------------------
// conversions between FP64 components and a column's fixed-point units

// ceil(log2 r): the growth bound (in bits) of a radix-r sub-stage
__host__ __device__ constexpr int fx_l(int r) {
  int l = 0;
  while ((1 << l) < r) ++l;
  return l;
}
// headroom bits of a pass whose first sub-stage has radix r0: every input
// component is below 2^B
__host__ __device__ constexpr int fx_b0(int r0) { return 61 - fx_l(r0) < 60 ? 61 - fx_l(r0) : 60; }
// a value's units divided by 2^s after a sub-stage (magnitude bound kept)
__device__ __forceinline__ Fx fx_shr(Fx v, int s) { return Fx::raw(v.v >> s); }
// biased exponent field, at least 1 (zero and subnormals count as 1)
__device__ __forceinline__ int fx_expo(double x) {
  const int e = (__double2hiint(x) >> 20) & 0x7ff;
  return e > 1 ? e : 1;
}
// round(x * 2^K) (half up) for a column whose exponent field maximum is E:
// x = m 2^(e - 1075) with the signed 53-bit significand m, so x 2^K =
// m / 2^t with t = 1075 - K - e = (53 - B) + (E - e), passed as cin - e with
// cin = 53 - B + E: a left shift (exact) when t <= 0, else rounded as
// floor((2m + 1) / 2^(t + 1))
__device__ __forceinline__ Fx fx_in(double x, int cin) {
  const long long b = __double_as_longlong(x);
  const int hi = (int)(b >> 32);
  const int e = (hi >> 20) & 0x7ff;
  long long m = (b & 0x000fffffffffffffll) | (e ? (1ll << 52) : 0ll);
  if (hi < 0) m = -m;
  const int t = cin - (e > 1 ? e : 1);
  if (t <= 0) return Fx::raw(m << -t);
  const int sh = t < 62 ? t + 1 : 63;
  return Fx::raw((2 * m + 1) >> sh);
}
constexpr int kFxNaN = -0x40000000;  // K of a column that held Inf or NaN

// v * 2^-K for results outside the normal double range (and NaN columns)
static __device__ __noinline__ double fx_out_rare(long long v, int K) {
  if (K == kFxNaN) return __longlong_as_double(0x7ff8000000000000ll);
  return ldexp((double)v, -K);
}
// v * 2^-K as a double, rounded to nearest (ties to even), from the
// integer's bits
__device__ __forceinline__ double fx_out(Fx v, int K) {
  const long long x = v.v;
  if (x == 0) return K == kFxNaN ? __longlong_as_double(0x7ff8000000000000ll) : 0.0;
  const unsigned long long sign = (unsigned long long)x & 0x8000000000000000ull;
  unsigned long long a = (unsigned long long)(x < 0 ? -x : x);
  const int lz = __clzll((long long)a);
  const int ef = 1086 - lz - K;  // exponent field of the result: 63 - lz - K + 1023
  if (ef <= 0 || ef >= 2047 || K == kFxNaN) return fx_out_rare(x, K);
  a <<= lz;                                   // leading one at bit 63
  unsigned long long m = a >> 11;             // 53 bits, leading one at bit 52
  const unsigned rem = (unsigned)a & 0x7ffu;  // the 11 bits dropped
  m += (rem > 0x400u || (rem == 0x400u && (m & 1ull))) ? 1ull : 0ull;
  // (ef - 1) << 52 plus m (with its leading one) carries into the exponent;
  // a rounding to 2^53 carries once more
  return __longlong_as_double((long long)(sign | (((unsigned long long)(ef - 1) << 52) + m)));
}
// the scale factor K of a column's inputs from its exponent maximum E
__device__ __forceinline__ int fx_k(int B, int E) { return E >= 2047 ? kFxNaN : B + 1022 - E; }

}  // namespace fftj
