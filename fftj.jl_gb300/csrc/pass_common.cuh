// Device building blocks of the pass kernels, shared by kernels.cu (the
// generic pass) and recipes.cu (passes specialised at compile time).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "bfly_consts.h"
#include "fftj_internal.h"
#include "fx64.cuh"

namespace fftj {

template <typename T>
struct CT;
template <>
struct CT<float> { using t = float2; };
template <>
struct CT<double> { using t = double2; };
template <>
struct CT<Fx> { using t = Fx2; };

template <typename T>
using Cx = typename CT<T>::t;

// Element type of the data in HBM for a pass that computes in T: the
// ComplexF64 passes compute in block fixed point (Fx, fx64.cuh) on FP64 data.
template <typename T>
struct HbmT { using t = T; };
template <>
struct HbmT<Fx> { using t = double; };
template <typename T>
using Hs = typename HbmT<T>::t;
template <typename T>
constexpr bool kFx = std::is_same<T, Fx>::value;

// read-only load of a table entry (twiddles: Q61 int64 pairs for Fx)
template <typename T>
__device__ __forceinline__ Cx<T> ldt(const Cx<T>* p) {
  if constexpr (kFx<T>) {
    const longlong2 v = __ldg(reinterpret_cast<const longlong2*>(p));
    Fx2 r;
    r.x = Fx::raw(v.x);
    r.y = Fx::raw(v.y);
    return r;
  } else {
    return __ldg(p);
  }
}

// ---- per-column conversion of Fx passes (no-ops for float and double).
// hexpo: the exponent field maximum of an element; to_c: HBM element ->
// compute element given cin = 53 - B + E of its column.
template <typename T>
__device__ __forceinline__ int hexpo(const Cx<Hs<T>>& h) {
  if constexpr (kFx<T>) {
    const int a = fx_expo(h.x), b = fx_expo(h.y);
    return a > b ? a : b;
  } else {
    return 0;
  }
}
template <typename T>
__device__ __forceinline__ Cx<T> to_c(const Cx<Hs<T>>& h, int cin) {
  if constexpr (kFx<T>) {
    Fx2 r;
    r.x = fx_in(h.x, cin);
    r.y = fx_in(h.y, cin);
    return r;
  } else {
    (void)cin;
    return h;
  }
}
// outputs of a sub-stage scaled down by 2^s for the next one (Fx only)
template <typename T>
__device__ __forceinline__ Cx<T> shr_c(Cx<T> v, int s) {
  if constexpr (kFx<T>) {
    v.x = fx_shr(v.x, s);
    v.y = fx_shr(v.y, s);
  }
  return v;
}
// growth bound in bits of the sub-stage after the first of Rs (0: none)
template <int r, int... rest>
__host__ __device__ constexpr int next_shift() {
  if constexpr (sizeof...(rest) > 0) {
    constexpr int a[] = {rest...};
    return fx_l(a[0]);
  } else {
    return 0;
  }
}

// largest exponent field of each tile column, combined across the lanes of
// a warp that share a column (one shared-memory atomic per column and warp)
__device__ __forceinline__ void col_expo_max(int* colE, int c, int e) {
  const unsigned act = __activemask();
  const unsigned grp = __match_any_sync(act, c);
  const int m = (int)__reduce_max_sync(grp, (unsigned)e);
  if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(colE + c, m);
}
// The store conversion and scaling of a pass: float/double multiply by the
// plan's scale when it is not 1; Fx converts back from the column's units,
// folding a power-of-two scale into the exponent shift.
template <typename T>
struct OutConv {
  bool scaled;
  T sc;
  __device__ __forceinline__ explicit OutConv(const PassParams& pp) {
    scaled = __double_as_longlong(pp.scale) != 0x3FF0000000000000ll;
    sc = (T)pp.scale;
  }
  __device__ __forceinline__ Cx<T> operator()(Cx<T> x, int /*E*/) const {
    if (scaled) { x.x *= sc; x.y *= sc; }
    return x;
  }
};
template <>
struct OutConv<Fx> {
  int B, se;   // headroom bits of the inputs; power-of-two part of the scale minus the stage shifts
  bool mul;    // the scale is not a positive power of two: multiply by its significand
  Fx sm;       // the significand as Q61, |sm| in [1/2, 1) (0 for a zero scale)
  __device__ __forceinline__ explicit OutConv(const PassParams& pp) {
    const long long b = __double_as_longlong(pp.scale);
    const long long frac = b & 0x000fffffffffffffll;
    const int field = (int)((b >> 52) & 0x7ff);
    B = pp.fx_b0;
    if (field == 0) {  // zero (or subnormal) scale: every output is 0
      mul = true;
      sm = Fx::raw(0);
      se = 0;
    } else if (frac == 0 && b > 0) {  // 2^(field - 1023): folded into the exponent
      mul = false;
      sm = Fx::raw(0);
      se = field - 1023;
    } else {  // +-(1 + frac/2^52)/2 * 2^(field - 1022)
      mul = true;
      const long long q = ((1ll << 52) | frac) << 8;
      sm = Fx::raw(b < 0 ? -q : q);
      se = field - 1022;
    }
    se += pp.fx_sht;  // values were divided by 2^fx_sht between sub-stages
  }
  __device__ __forceinline__ double2 operator()(Fx2 x, int E) const {
    int K = fx_k(B, E);
    if (K != kFxNaN) K -= se;  // se includes the sub-stage shifts
    if (mul) {
      x.x = sm * x.x;
      x.y = sm * x.y;
    }
    double2 r;
    r.x = fx_out(x.x, K);
    r.y = fx_out(x.y, K);
    return r;
  }
};
template <typename T>
__device__ __forceinline__ Cx<T> mk(T x, T y) { Cx<T> c; c.x = x; c.y = y; return c; }
template <typename C>
__device__ __forceinline__ C add(C a, C b) { C c; c.x = a.x + b.x; c.y = a.y + b.y; return c; }
template <typename C>
__device__ __forceinline__ C sub(C a, C b) { C c; c.x = a.x - b.x; c.y = a.y - b.y; return c; }
// a * w (complex)
template <typename C>
__device__ __forceinline__ C cmul(C a, C w) {
  C c;
  c.x = fma(w.x, a.x, -(w.y * a.y));
  c.y = fma(w.x, a.y, w.y * a.x);
  return c;
}
// (DIR * i) * z
template <int DIR, typename C>
__device__ __forceinline__ C mul_di(C z) {
  C c;
  if (DIR < 0) { c.x = z.y; c.y = -z.x; } else { c.x = -z.y; c.y = z.x; }
  return c;
}

// Load of transform data. Kernels read their inputs through the read-only
// path (__ldg); the persistent group kernel reads data that other CTAs of
// the same launch wrote, so it uses L2-coherent loads (__ldcg) instead.
template <bool CG, typename V>
__device__ __forceinline__ V ldd(const V* p) {
  if constexpr (CG) return __ldcg(p);
  else return __ldg(p);
}

// Predicates and factors from double kernel parameters, formed with integer
// operations on the double's bits. A floating compare or conversion of a
// double parameter that the compiler re-evaluates per element (it does, to
// spare predicate registers) runs on the FP64 pipe, 1/64 of the FP32 rate on
// GB300: in an F32 pass that kept the FP64 pipe 47% busy.
__device__ __forceinline__ bool not_one(double x) { return __double_as_longlong(x) != 0x3FF0000000000000ll; }
template <typename T>
__device__ __forceinline__ T half_or_one(double x) { return not_one(x) ? (T)0.5 : (T)1; }

// Shared-memory padding: one element per 16 (8-byte) or 8 (16-byte) elements,
// so power-of-two strides spread over the banks.
template <typename T>
__device__ __forceinline__ int pidx(int i) { return i + (i >> (sizeof(T) == 4 ? 4 : 3)); }

// ---------------------------------------------------------------------------
// Register DFTs (FFTJ src/kernels.jl:93-239: bf2, bf4_core, bf8_core, bfp).
template <typename T, int DIR>
__device__ __forceinline__ void dft4(Cx<T>& a, Cx<T>& b, Cx<T>& c, Cx<T>& d) {
  Cx<T> apc = add(a, c), amc = sub(a, c), bpd = add(b, d), bmd = mul_di<DIR>(sub(b, d));
  a = add(apc, bpd);
  c = sub(apc, bpd);
  b = add(amc, bmd);
  d = sub(amc, bmd);
}

template <typename T, int DIR, int R>
struct Dft;

template <typename T, int DIR>
struct Dft<T, DIR, 2> {
  __device__ __forceinline__ static void run(Cx<T>* v) {
    Cx<T> a = v[0];
    v[0] = add(a, v[1]);
    v[1] = sub(a, v[1]);
  }
};
template <typename T, int DIR>
struct Dft<T, DIR, 4> {
  __device__ __forceinline__ static void run(Cx<T>* v) { dft4<T, DIR>(v[0], v[1], v[2], v[3]); }
};
template <typename T, int DIR>
struct Dft<T, DIR, 8> {
  __device__ __forceinline__ static void run(Cx<T>* v) {
    Cx<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    Cx<T> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<T, DIR>(e0, e1, e2, e3);
    dft4<T, DIR>(o0, o1, o2, o3);
    const T c = (T)0.70710678118654752440;
    Cx<T> t1, t3;
    if (DIR < 0) {
      t1 = mk<T>(c * (o1.x + o1.y), c * (o1.y - o1.x));
      t3 = mk<T>(c * (o3.y - o3.x), -c * (o3.x + o3.y));
    } else {
      t1 = mk<T>(c * (o1.x - o1.y), c * (o1.y + o1.x));
      t3 = mk<T>(-c * (o3.x + o3.y), c * (o3.x - o3.y));
    }
    Cx<T> t2 = mul_di<DIR>(o2);
    v[0] = add(e0, o0); v[4] = sub(e0, o0);
    v[1] = add(e1, t1); v[5] = sub(e1, t1);
    v[2] = add(e2, t2); v[6] = sub(e2, t2);
    v[3] = add(e3, t3); v[7] = sub(e3, t3);
  }
};
template <typename T, int DIR>
struct Dft<T, DIR, 16> {
  __device__ __forceinline__ static void run(Cx<T>* v) {
    // 4 x 4: x[4 n1 + n2], X[k1 + 4 k2]
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) dft4<T, DIR>(v[n2], v[4 + n2], v[8 + n2], v[12 + n2]);
    // now v[4*k1 + n2] holds a_{n2}[k1]; twiddle by w16^(n2*k1)
#pragma unroll
    for (int k1 = 1; k1 < 4; ++k1)
#pragma unroll
      for (int n2 = 1; n2 < 4; ++n2) {
        const int t = n2 * k1;
        Cx<T> w = mk<T>((T)kCos16(t), (T)(DIR * kSin16(t)));
        v[4 * k1 + n2] = cmul(v[4 * k1 + n2], w);
      }
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4<T, DIR>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    // v[4*k1 + k2] holds X[k1 + 4 k2]: transpose to natural order
    Cx<T> o[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
      for (int k2 = 0; k2 < 4; ++k2) o[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = o[i];
  }
};

template <int P>
struct PrimeTab;
template <>
struct PrimeTab<3> { __device__ static constexpr double c(int i) { return kCos3(i); } __device__ static constexpr double s(int i) { return kSin3(i); } };
template <>
struct PrimeTab<5> { __device__ static constexpr double c(int i) { return kCos5(i); } __device__ static constexpr double s(int i) { return kSin5(i); } };
template <>
struct PrimeTab<7> { __device__ static constexpr double c(int i) { return kCos7(i); } __device__ static constexpr double s(int i) { return kSin7(i); } };
template <>
struct PrimeTab<11> { __device__ static constexpr double c(int i) { return kCos11(i); } __device__ static constexpr double s(int i) { return kSin11(i); } };
template <>
struct PrimeTab<13> { __device__ static constexpr double c(int i) { return kCos13(i); } __device__ static constexpr double s(int i) { return kSin13(i); } };

// odd prime P by conjugate pairs (FFTJ bfp, src/kernels.jl:146-228)
template <typename T, int DIR, int P>
struct DftPrime {
  __device__ __forceinline__ static void run(Cx<T>* v) {
    constexpr int h = (P - 1) / 2;
    Cx<T> t[h], d[h];
#pragma unroll
    for (int j = 1; j <= h; ++j) {
      t[j - 1] = add(v[j], v[P - j]);
      d[j - 1] = sub(v[j], v[P - j]);
    }
    Cx<T> x0 = v[0];
    Cx<T> sum = t[0];
#pragma unroll
    for (int j = 2; j <= h; ++j) sum = add(sum, t[j - 1]);
    v[0] = add(x0, sum);
#pragma unroll
    for (int k = 1; k <= h; ++k) {
      Cx<T> u = x0, w = mk<T>(0, 0);
#pragma unroll
      for (int j = h; j >= 1; --j) {
        const T c = (T)PrimeTab<P>::c((k - 1) * h + j - 1);
        const T s = (T)(DIR * PrimeTab<P>::s((k - 1) * h + j - 1));
        u.x = fma(c, t[j - 1].x, u.x);
        u.y = fma(c, t[j - 1].y, u.y);
        w.x = fma(s, d[j - 1].x, w.x);
        w.y = fma(s, d[j - 1].y, w.y);
      }
      v[k] = mk<T>(u.x - w.y, u.y + w.x);      // u + i w
      v[P - k] = mk<T>(u.x + w.y, u.y - w.x);  // u - i w
    }
  }
};
template <typename T, int DIR>
struct Dft<T, DIR, 3> { __device__ __forceinline__ static void run(Cx<T>* v) { DftPrime<T, DIR, 3>::run(v); } };
template <typename T, int DIR>
struct Dft<T, DIR, 5> { __device__ __forceinline__ static void run(Cx<T>* v) { DftPrime<T, DIR, 5>::run(v); } };
template <typename T, int DIR>
struct Dft<T, DIR, 7> { __device__ __forceinline__ static void run(Cx<T>* v) { DftPrime<T, DIR, 7>::run(v); } };
template <typename T, int DIR>
struct Dft<T, DIR, 11> { __device__ __forceinline__ static void run(Cx<T>* v) { DftPrime<T, DIR, 11>::run(v); } };
template <typename T, int DIR>
struct Dft<T, DIR, 13> { __device__ __forceinline__ static void run(Cx<T>* v) { DftPrime<T, DIR, 13>::run(v); } };

// ---------------------------------------------------------------------------
// One radix-r sub-stage of the run-time-radix pass between two shared
// buffers: the maps of substage<> (butterfly k = p S + q of column b reads
// k + j Rr, writes r S p + j S + q, twiddled by w_R^(p j S)), from src to
// dst. With the input and output apart, a thread runs its butterflies one
// at a time in a loop that is not unrolled: registers for r elements, and a
// small body per radix (no calls, no spills).
template <typename T, int DIR, int r>
__device__ __forceinline__ void substage_pp(const Cx<T>* __restrict__ src, Cx<T>* __restrict__ dst, const int b,
                                            const int kg, const int Tf, const int NB, const int Rr, const int S,
                                            const FastDiv fS, const Cx<T>* __restrict__ twR, const int sh,
                                            const bool raw = false, const int cin = 0) {
  const int jstride_in = Rr * NB;
  const int jstride_out = S * NB;
#pragma unroll 1
  for (int k = kg; k < Rr; k += Tf) {
    Cx<T> v[r];
    const int a = k * NB + b;
    if (kFx<T> && raw) {
      // first sub-stage of an Fx pass: the buffer holds the raw FP64 inputs
      // of column b, converted here with the column's scale
      const Cx<Hs<T>>* rs = reinterpret_cast<const Cx<Hs<T>>*>(src);
#pragma unroll
      for (int j = 0; j < r; ++j) v[j] = to_c<T>(rs[pidx<T>(a + j * jstride_in)], cin);
    } else {
#pragma unroll
      for (int j = 0; j < r; ++j) v[j] = src[pidx<T>(a + j * jstride_in)];
    }
    const int p = (int)fS.div((uint32_t)k);
    const int q = k - p * S;
    Dft<T, DIR, r>::run(v);
    const int ao = (r * S * p + q) * NB + b;
    dst[pidx<T>(ao)] = shr_c<T>(v[0], sh);
    const int tstep = p * S;
#pragma unroll
    for (int j = 1; j < r; ++j) {
      Cx<T> w = v[j];
      if (p != 0) w = cmul(w, ldt<T>(&twR[j * tstep]));
      dst[pidx<T>(ao + j * jstride_out)] = shr_c<T>(w, sh);
    }
  }
}

// LOADOP = LOAD_RUNTIME reads the load op from pp (one code path for all;
// the group kernel uses it to keep its instantiation count small).
constexpr int LOAD_RUNTIME = -1;

// twiddle of the irfft pre-pass: one table w[g] (g < h), or for long
// halves the two-level product hi[g >> sh] * lo[g & (2^sh - 1)] of two
// L1/L2-resident tables (the single table would stream from HBM beside the
// data)
template <typename T>
__device__ __forceinline__ Cx<T> c2r_twiddle(const PassParams& pp, int64_t g) {
  if (pp.ld_sh) {
    const Cx<T> hi = __ldg(reinterpret_cast<const Cx<T>*>(pp.ld_tab) + (g >> pp.ld_sh));
    const Cx<T> lo = __ldg(reinterpret_cast<const Cx<T>*>(pp.ld_tab2) + (g & ((1ll << pp.ld_sh) - 1)));
    return cmul(hi, lo);
  }
  return __ldg(reinterpret_cast<const Cx<T>*>(pp.ld_tab) + g);
}

// irfft pre-pass of one entry (FFTJ src/real.jl:149-192): Z = xe + i (w xd)
// from a = X[g], its mirror bb = X[h - g] and the twiddle w = w_n^g
template <typename T>
__device__ __forceinline__ Cx<T> c2r_pre_combine(Cx<T> a, Cx<T> bb, Cx<T> w, T pre) {
  bb.y = -bb.y;
  const Cx<T> xe = mk<T>((a.x + bb.x) * pre, (a.y + bb.y) * pre);
  const Cx<T> xd = mk<T>((a.x - bb.x) * pre, (a.y - bb.y) * pre);
  const T tr = fma(w.x, xd.x, -(w.y * xd.y));
  const T ti = fma(w.x, xd.y, w.y * xd.x);
  return mk<T>(xe.x - ti, xe.y + tr);
}

template <typename T, int LOADOP, bool CG = false>
__device__ __forceinline__ Cx<T> load_elem(const PassParams& pp, const void* in, int64_t b, int64_t g);

template <typename T, bool CG>
__device__ __forceinline__ Cx<T> load_elem_rt(const PassParams& pp, const void* in, int64_t b, int64_t g) {
  switch (pp.load_op) {
    case LOAD_DECONV: return load_elem<T, LOAD_DECONV, CG>(pp, in, b, g);
    case LOAD_SPREAD: return load_elem<T, LOAD_SPREAD, CG>(pp, in, b, g);
    case LOAD_C2R_PRE: return load_elem<T, LOAD_C2R_PRE, CG>(pp, in, b, g);
    case LOAD_REAL: return load_elem<T, LOAD_REAL, CG>(pp, in, b, g);
    default: return load_elem<T, LOAD_PLAIN, CG>(pp, in, b, g);
  }
}

template <typename T, int LOADOP, bool CG>
__device__ __forceinline__ Cx<T> load_elem(const PassParams& pp, const void* in, int64_t b, int64_t g) {
  if constexpr (LOADOP == LOAD_RUNTIME) return load_elem_rt<T, CG>(pp, in, b, g);
  if (LOADOP == LOAD_PLAIN) {
    return ldd<CG>(reinterpret_cast<const Cx<T>*>(in) + b * pp.in_bstride + g);
  } else if (LOADOP == LOAD_DECONV) {
    // grid position g of the length-m zero-padded deconvolved input
    // (FFTJ _deconv! + zero fill, src/resample.jl:258-301); along a strided
    // N-d axis g = a * inner + i (RsPass lanes, src/resample.jl:511-536)
    const int64_t n = pp.ld_n, m = pp.ld_m, hp = pp.ld_hp, inner = pp.ld_inner > 1 ? pp.ld_inner : 1;
    int64_t a = g, i = 0;
    if (inner > 1) { a = g / inner; i = g - a * inner; }
    int64_t j;
    if (a < hp) j = a;
    else if (a >= m - n + hp) j = a - (m - n);
    else return mk<T>(0, 0);
    const Cx<T> x = ldd<CG>(reinterpret_cast<const Cx<T>*>(in) + b * pp.ld_stride + j * inner + i);
    const T c = __ldg(reinterpret_cast<const T*>(pp.ld_tab) + j);
    return mk<T>(x.x * c, x.y * c);
  } else if (LOADOP == LOAD_SPREAD) {
    // HvdH Gaussian spread (src/hvdh.jl:355-470, per output row as the
    // batched HvPass): grid row a = sum_o wt[a*w + o] * x[(l0[a] + o) mod n];
    // along a strided axis (HvPass lanes, src/hvdh.jl:696-702) g = a * inner
    // + i and input row r of lane i sits at r * inner + i
    const int64_t n = pp.ld_n, inner = pp.ld_inner > 1 ? pp.ld_inner : 1;
    int64_t a = g, i = 0;
    if (inner > 1) { a = g / inner; i = g - a * inner; }
    const int w = pp.ld_w;
    const Cx<T>* x = reinterpret_cast<const Cx<T>*>(in) + b * pp.ld_stride + i;
    const T* wt = reinterpret_cast<const T*>(pp.ld_tab) + a * w;
    int64_t r = __ldg(pp.ld_l0 + a);
    T re = 0, im = 0;
    for (int o = 0; o < w; ++o) {
      const T c = __ldg(wt + o);
      const Cx<T> v = ldd<CG>(x + r * inner);
      re = fma(c, v.x, re);
      im = fma(c, v.y, im);
      if (++r == n) r = 0;
    }
    return mk<T>(re, im);
  } else if (LOADOP == LOAD_C2R_PRE) {
    // irfft pre-pass (FFTJ src/real.jl:149-192): Z[k] = xe + i (w xd)
    const int64_t h = pp.ld_n;
    const Cx<T>* X = reinterpret_cast<const Cx<T>*>(in) + b * pp.ld_stride;
    const Cx<T> a = ldd<CG>(X + g);
    Cx<T> bb = ldd<CG>(X + (h - g));
    bb.y = -bb.y;
    const T pre = half_or_one<T>(pp.ld_pre);  // 1/2 (irfft) or 1 (brfft)
    const Cx<T> xe = mk<T>((a.x + bb.x) * pre, (a.y + bb.y) * pre);
    const Cx<T> xd = mk<T>((a.x - bb.x) * pre, (a.y - bb.y) * pre);
    const Cx<T> w = c2r_twiddle<T>(pp, g);
    const T tr = fma(w.x, xd.x, -(w.y * xd.y));
    const T ti = fma(w.x, xd.y, w.y * xd.x);
    return mk<T>(xe.x - ti, xe.y + tr);
  } else {  // LOAD_REAL
    const T x = ldd<CG>(reinterpret_cast<const T*>(in) + b * pp.ld_stride + g);
    return mk<T>(x, 0);
  }
}

template <typename T>
__device__ __forceinline__ Cx<T> outer_tw(const PassParams& pp, int64_t e) {
  if (pp.tw_mode == 1) return ldt<T>(reinterpret_cast<const Cx<T>*>(pp.tw_full) + e);
  const Cx<T> hi = ldt<T>(reinterpret_cast<const Cx<T>*>(pp.tw_hi) + (e >> pp.tw_shift));
  const Cx<T> lo = ldt<T>(reinterpret_cast<const Cx<T>*>(pp.tw_lo) + (e & ((1ll << pp.tw_shift) - 1)));
  Cx<T> w = cmul(hi, lo);
  if constexpr (kFx<T>) {
    // the rounded product of two Q61 twiddles can land a few units beyond
    // +-(2^61 - 1) (at angles near multiples of pi/2): clamp to the Q61 range
    w.x = fx_clamp_q61(w.x);
    w.y = fx_clamp_q61(w.y);
  }
  return w;
}

// ---------------------------------------------------------------------------
// Passes specialised at compile time: the radix sequence of the pass's
// R-point DFT is a template parameter pack, so R, the sub-stage strides S and
// the threads per column are constants and every index is strength-reduced.
struct RuntimeRecipe {
  static constexpr bool kConst = false;
  static constexpr int R = 1;
  static constexpr int Tf = 1;
};

template <int... Rs>
struct Recipe {
  static constexpr bool kConst = true;
  static constexpr int n = sizeof...(Rs);
  static constexpr int R = (Rs * ... * 1);
  // threads per column: the smallest count with <= 16 elements per thread and
  // <= max(1, 16/r) butterflies per thread in every sub-stage (the host
  // planner applies the same rule)
  static constexpr int tf() {
    constexpr int a[] = {Rs...};
    for (int t = 1; t <= R; ++t) {
      bool ok = (R + t - 1) / t <= 16;
      for (int i = 0; i < n && ok; ++i) {
        const int cap = 16 / a[i] > 0 ? 16 / a[i] : 1;
        if ((R / a[i] + t - 1) / t > cap) ok = false;
      }
      if (ok) return t;
    }
    return R;
  }
  static constexpr int Tf = tf();
};

// compile-time sub-stage: the maps of substage<> with constant r, S, R/r, Tf
// Padded index of x + j*J: when J is a multiple of the padding period,
// pidx(x + j J) = pidx(x) + j (J + J / period), so a butterfly's accesses are
// one base index plus constant steps (no per-access shift and add).
template <typename T>
__host__ __device__ constexpr int pad_period() { return sizeof(T) == 4 ? 16 : 8; }

// Tile positions when the tile's column count is a compile-time constant
// NBC: element (row, column b < NBC) sits at pidx(row * NBC + b), computed
// as a row part plus a column part, so that two rows a fixed distance apart
// are a constant offset apart (immediate shared-memory offsets instead of a
// shift and adds per access). NBC divides the padding period or is a
// multiple of it.
template <typename T, int NBC>
struct Lay {
  static constexpr int PP = pad_period<T>();
  static_assert(NBC > 0 && (PP % NBC == 0 || NBC % PP == 0), "column count must divide the padding period or be a multiple of it");
  static constexpr int RP = NBC >= PP ? 1 : PP / NBC;  // rows per padding period (a power of two)
  static constexpr int LS = RP == 1 ? 0 : RP == 2 ? 1 : RP == 4 ? 2 : RP == 8 ? 3 : 4;
  __device__ __forceinline__ static int col(int b) { return NBC >= PP ? b + b / PP : b; }
  __device__ __forceinline__ static int row(int r) { return NBC >= PP ? r * (NBC + NBC / PP) : r * NBC + (r >> LS); }
  // row(r0 + d) - row(r0): exact when d or r0 is a multiple of RP
  __host__ __device__ static constexpr int step(int d) { return NBC >= PP ? d * (NBC + NBC / PP) : d * NBC + d / RP; }
  __host__ __device__ static constexpr bool exact(int d) { return d % RP == 0; }
};
// the layout of NBC columns, or a placeholder when the count is a run-time
// value (NBC == 0; the callers then take the pidx path)
template <typename T, int NBC>
using LayC = Lay<T, NBC == 0 ? 1 : NBC>;

template <typename T, int DIR, int r, int S, int Rr, int TF, int NBC = 0, int SH = 0>
__device__ __forceinline__ void substage_ct(Cx<T>* __restrict__ buf, const int b, const int kg, const int NB,
                                            const Cx<T>* __restrict__ twR) {
  constexpr int IPT = (Rr + TF - 1) / TF;
  constexpr int PP = pad_period<T>();
  const int jstride_in = Rr * NB;
  const int jstride_out = S * NB;
  Cx<T> v[IPT][r];
#pragma unroll
  for (int i = 0; i < IPT; ++i) {
    const int k = kg + i * TF;
    if ((i + 1) * TF <= Rr || k < Rr) {
      const int a = k * NB + b;
      if constexpr (NBC > 0 && LayC<T, NBC>::exact(Rr)) {
        const int base = LayC<T, NBC>::row(k) + LayC<T, NBC>::col(b);
#pragma unroll
        for (int j = 0; j < r; ++j) v[i][j] = buf[base + j * LayC<T, NBC>::step(Rr)];
      } else if constexpr (Rr % PP == 0) {
        const int base = pidx<T>(a), step = jstride_in + jstride_in / PP;
#pragma unroll
        for (int j = 0; j < r; ++j) v[i][j] = buf[base + j * step];
      } else {
#pragma unroll
        for (int j = 0; j < r; ++j) v[i][j] = buf[pidx<T>(a + j * jstride_in)];
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < IPT; ++i) {
    const int k = kg + i * TF;
    if ((i + 1) * TF <= Rr || k < Rr) {
      const int p = k / S;
      const int q = k - p * S;
      Dft<T, DIR, r>::run(v[i]);
      const int a = (r * S * p + q) * NB + b;
      // compile-time columns: rows r S p + q + j S are constant offsets apart
      // when S is a multiple of the rows per padding period, or S == 1 and r
      // is (then the first row r p is one)
      constexpr bool kLay = NBC > 0 && (LayC<T, NBC>::exact(S) || (S == 1 && LayC<T, NBC>::exact(r)));
      const int base = kLay ? LayC<T, NBC>::row(r * S * p + q) + LayC<T, NBC>::col(b) : pidx<T>(a);
      const int step = (S % PP == 0) ? jstride_out + jstride_out / PP : 0;
      // position of output j: a constant step when S is a multiple of the
      // padding period, else the padded index of a + j * S * NB
#define FFTJ_OUT_AT(j)                                                               \
  (kLay ? base + LayC<T, NBC>::step((j) * S)                           \
        : (S % PP == 0) ? base + (j) * step : pidx<T>(a + (j) * jstride_out))
      buf[base] = shr_c<T>(v[i][0], SH);
      if (Rr == S) {
        // last sub-stage of the pass (L = r): no twiddle
#pragma unroll
        for (int j = 1; j < r; ++j) buf[FFTJ_OUT_AT(j)] = shr_c<T>(v[i][j], SH);
      } else {
        const int tstep = p * S;
#pragma unroll
        for (int j = 1; j < r; ++j) {
          Cx<T> w = v[i][j];
          if (p != 0) w = cmul(w, twR[j * tstep]);
          buf[FFTJ_OUT_AT(j)] = shr_c<T>(w, SH);
        }
      }
#undef FFTJ_OUT_AT
    }
  }
  __syncthreads();
}

template <typename T, int DIR, int TF, int R, int S, int NBC, int r, int... rest>
__device__ __forceinline__ void run_subs_ct(Cx<T>* buf, const int b, const int kg, const int NB,
                                            const Cx<T>* twR) {
  substage_ct<T, DIR, r, S, R / r, TF, NBC, next_shift<r, rest...>()>(buf, b, kg, NB, twR);
  if constexpr (sizeof...(rest) > 0) run_subs_ct<T, DIR, TF, R, S * r, NBC, rest...>(buf, b, kg, NB, twR);
}
template <typename T, int DIR, int... Rs>
__device__ __forceinline__ void run_recipe(Recipe<Rs...>*, Cx<T>* buf, const int b, const int kg, const int NB,
                                           const Cx<T>* twR) {
  run_subs_ct<T, DIR, Recipe<Rs...>::Tf, Recipe<Rs...>::R, 1, 0, Rs...>(buf, b, kg, NB, twR);
}

// ---------------------------------------------------------------------------
// Precision form of a radix-16 sub-stage (F32 passes, plan option
// precision = 1 FP16 / 2 BF16): the 16-point DFTs of the whole tile as one
// GEMM on the tensor cores. In real form a butterfly's outputs are
// [Yr; Yi] = [[Cr, -Ci], [Ci, Cr]] [Xr; Xi] (32 x 32 times 32 x 1); a warp
// multiplies it into n-tiles of 8 butterflies with mma.sync m16n8k16
// (half-precision operands, FP32 accumulation). Operands are split into a
// hi half and a lo half scaled up by 2^11 (FP16) or 2^8 (BF16) so that it
// never goes subnormal; A_hi B_hi accumulates in one accumulator and
// A_hi B_lo + A_lo B_hi in another, which is scaled back down (the lo*lo
// product is dropped). Each butterfly (a GEMM column) is scaled by its own
// power of two so that its largest input is below 1 (FP16 range) and
// unscaled on the way out. Outputs get the sub-stage's twiddles in FP32 and
// go to the same places as the FP32 sub-stage's.
template <int KIND>  // 1: FP16 operands, 2: BF16 operands
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
  if constexpr (KIND == 1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
  } else {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
  }
}

// lo halves are stored multiplied by kLoScale (2^mantissa bits of the half
// type), so they stay normal numbers
template <int KIND>
__host__ __device__ constexpr float lo_scale() { return KIND == 1 ? 2048.f : 256.f; }

// (x, y) -> packed hi halves and packed scaled lo halves
template <int KIND>
__device__ __forceinline__ void split_pair(float x, float y, uint32_t& hi, uint32_t& lo) {
  constexpr float L = lo_scale<KIND>();
  if constexpr (KIND == 1) {
    const __half2 h = __floats2half2_rn(x, y);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn((x - hf.x) * L, (y - hf.y) * L);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  } else {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x, y);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn((x - hf.x) * L, (y - hf.y) * L);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
  }
}

// Whether the tensor-core sub-stage applies: whole warps, butterflies in
// n-tiles of 8, at most 4 n-tiles per warp (EPT <= 16 guarantees it).
__device__ __forceinline__ bool tc16_fits(int nthr, int NB, int Rr) {
  const int nbf = NB * Rr;
  return (nthr & 31) == 0 && (nbf & 7) == 0 && (nbf >> 3) <= 4 * (nthr >> 5);
}

template <int DIR, int KIND>
__device__ __noinline__ void substage_tc16(float2* __restrict__ buf, const int tid, const int nthr, const int NB,
                                           const int Rr, const int S, const FastDiv fS, const FastDiv fNB,
                                           const float2* __restrict__ twR) {
  const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
  const bool active = tid < nthr;
  const int ntiles = (NB * Rr) >> 3;
  const int g = lane >> 2, j0 = (lane & 3) * 2;
  const int jstride = Rr * NB;
  // ---- inputs X[j0], X[j0+1], X[j0+8], X[j0+9] of butterfly 8 tile + g
  float xr[4][4], xi[4][4];
  int ex[4];  // exponent of each n-tile's butterfly g: |x| < 2^ex
#pragma unroll
  for (int it = 0; it < 4; ++it) {
    const int tile = warp + it * nwarps;
    float mx = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      xr[it][q] = 0.f;
      xi[it][q] = 0.f;
    }
    if (active && tile < ntiles) {
      const int u = tile * 8 + g;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = j0 + (q & 1) + (q >> 1) * 8;
        const float2 v = buf[pidx<float>(u + j * jstride)];
        xr[it][q] = v.x;
        xi[it][q] = v.y;
        mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
      }
    }
    // the four lanes 4g .. 4g+3 hold butterfly g's 16 inputs
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
    ex[it] = 0;
    if (mx > 0.f) frexpf(mx, &ex[it]);
  }
  __syncthreads();  // every input is in registers before any output is written
  // ---- DFT matrix fragments (row block mt: 0 = Yr, 1 = Yi; column block
  // kt: 0 = Xr, 1 = Xi), split into hi and scaled lo
  // A thread's entries are w_16^(row col) for row in {g, g+8} and col in
  // {j0, j0+1, j0+8, j0+9}: two roots w_16^(g j0), w_16^(g (j0+1)) and sign
  // flips, since w_16^8 = -1 and (g + 8 dr)(c + 8 dc) = g c + 8 (dr c + dc g)
  // modulo 16.
  float wc[2], ws[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float sn, cs;
    sincospif((float)((g * (j0 + h)) & 15) * 0.125f, &sn, &cs);
    wc[h] = cs;
    ws[h] = DIR * sn;
  }
  uint32_t ahi[2][2][4], alo[2][2][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int kt = 0; kt < 2; ++kt)
#pragma unroll
      for (int rg = 0; rg < 4; ++rg) {
        // register rg holds elements (row, col) and (row, col + 1),
        // row = g + 8 dr, col = j0 + 8 dc
        const int dr = rg & 1, dc = rg >> 1;
        float val[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float sg = ((dr * (j0 + h) + dc * g) & 1) ? -1.f : 1.f;
          const float cr = sg * wc[h], ci = sg * ws[h];
          val[h] = mt == 0 ? (kt == 0 ? cr : -ci) : (kt == 0 ? ci : cr);
        }
        split_pair<KIND>(val[0], val[1], ahi[mt][kt][rg], alo[mt][kt][rg]);
      }
  constexpr float kInvLo = 1.f / lo_scale<KIND>();
  // ---- products and outputs
#pragma unroll
  for (int it = 0; it < 4; ++it) {
    const int tile = warp + it * nwarps;
    if (!active || tile >= ntiles) continue;  // warp-uniform
    const float scale = ldexpf(1.f, -ex[it]);
    uint32_t bhi[2][2], blo[2][2];
    split_pair<KIND>(xr[it][0] * scale, xr[it][1] * scale, bhi[0][0], blo[0][0]);
    split_pair<KIND>(xr[it][2] * scale, xr[it][3] * scale, bhi[0][1], blo[0][1]);
    split_pair<KIND>(xi[it][0] * scale, xi[it][1] * scale, bhi[1][0], blo[1][0]);
    split_pair<KIND>(xi[it][2] * scale, xi[it][3] * scale, bhi[1][1], blo[1][1]);
    float acc[2][4], accl[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[mt][c] = accl[mt][c] = 0.f;
#pragma unroll
      for (int kt = 0; kt < 2; ++kt) {
        mma16816<KIND>(acc[mt], ahi[mt][kt], bhi[kt]);
        mma16816<KIND>(accl[mt], ahi[mt][kt], blo[kt]);
        mma16816<KIND>(accl[mt], alo[mt][kt], bhi[kt]);
      }
    }
    // the unscale exponents of the output butterflies j0 and j0 + 1 live in
    // lanes 4 j0 and 4 (j0 + 1)
    const int e0 = __shfl_sync(0xffffffffu, ex[it], j0 * 4);
    const int e1 = __shfl_sync(0xffffffffu, ex[it], j0 * 4 + 4);
    // accumulator c holds output row g + 8 (c >> 1) of butterfly
    // 8 tile + j0 + (c & 1)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int m = g + (c >> 1) * 8;
      const int u = tile * 8 + j0 + (c & 1);
      const int k = (int)fNB.div((uint32_t)u);
      const int bcol = u - k * NB;
      const int p = (int)fS.div((uint32_t)k);
      const int q = k - p * S;
      const float un = ldexpf(1.f, (c & 1) ? e1 : e0);
      float2 y = make_float2(fmaf(accl[0][c], kInvLo, acc[0][c]) * un, fmaf(accl[1][c], kInvLo, acc[1][c]) * un);
      if (p != 0 && m != 0) y = cmul(y, twR[m * p * S]);
      buf[pidx<float>((16 * S * p + m * S + q) * NB + bcol)] = y;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// One Stockham pass over one tile with the radix sequence read at run time
// from pp.sub: the generic kernel (k_pass) and the persistent group kernel.
// Compile-time recipes run pass_fused. The maps are those of the kernel
// comment in kernels.cu.
//
// The tile ping-pongs between two shared buffers. Loads stream into the
// first buffer -- for Fx passes the raw FP64 values, converted when the
// first sub-stage reads them, once every column's exponent maximum is
// known; every sub-stage reads one buffer and writes the other, one
// butterfly at a time; the store streams the result out with the outer
// twiddle and the scale. No phase keeps more than a few elements per thread
// in registers.
//
// pass_tile runs tile `tile` with threads [0, nthr) of the CTA doing the
// work. GROUP (the persistent group kernel): the CTA may have more threads
// than the pass (the extra ones only join the barriers), and data loads are
// L2-coherent.
template <typename T, int DIR, int LOADOP, class Rec, bool GROUP>
__device__ __forceinline__ void pass_tile(const PassParams& pp, const void* __restrict__ in,
                                          Cx<Hs<T>>* __restrict__ out, const uint32_t tile, const int tid,
                                          const int nthr) {
  static_assert(!Rec::kConst, "compile-time recipes run pass_fused");
  using H = Hs<T>;
  static_assert(sizeof(Cx<H>) == sizeof(Cx<T>), "raw and compute elements share the tile layout");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* const bufA = reinterpret_cast<Cx<T>*>(smem_raw);
  Cx<T>* const bufB = bufA + pp.smem_elems;
  int* const colE = reinterpret_cast<int*>(bufA + 2 * pp.smem_elems);
  const bool active = !GROUP || tid < nthr;
  const uint32_t t1 = pp.ftq.div(tile);
  const uint32_t tq = tile - t1 * pp.tiles_q;
  const uint32_t tb = pp.ftp.div(t1);
  const uint32_t tp = t1 - tb * pp.tiles_p;
  const int64_t q0 = (int64_t)tq * pp.Q, p0 = (int64_t)tp * pp.P, b0 = (int64_t)tb * pp.NBt;
  const int R = pp.R, Tf = pp.Tf;
  const int P = pp.P, Q = pp.Q, NB = pp.NB;
  const int E = active ? NB * R : 0;  // idle threads own no elements
  const int64_t ms = pp.m * pp.s;
  // this thread's column b = (bt, pl, ql) and first butterfly row kg (idle
  // threads get a row beyond every sub-stage, so they own no butterflies)
  const int kg = active ? (int)pp.fNB.div((uint32_t)tid) : (1 << 29);
  const int b = active ? tid - kg * NB : 0;
  const int cq = (int)pp.fQ.div((uint32_t)b);
  const int ql = b - cq * Q;
  const int cbt = (int)pp.fP.div((uint32_t)cq);
  const int pl = cq - cbt * P;
  const int64_t batch = b0 + cbt;
  const int64_t pcol = p0 + pl;
  const int B = pp.fx_b0;
  Cx<H>* const rawA = reinterpret_cast<Cx<H>*>(bufA);

  // ---- load: HBM -> first buffer, element by element
  if constexpr (kFx<T>) {
    if (tid < NB) colE[tid] = 1;
    __syncthreads();
  }
  if (pp.load_rows) {
    // transforms contiguous along j (one pass over whole transforms)
#pragma unroll 4
    for (int e = tid; e < E; e += nthr) {
      const int c = (int)pp.fR.div((uint32_t)e);
      const int j = e - c * R;
      const int64_t bb = b0 + c;
      const Cx<H> v = bb < pp.nbatch ? load_elem<H, LOADOP, GROUP>(pp, in, bb, j) : mk<H>(0, 0);
      if constexpr (kFx<T>) col_expo_max(colE, c, hexpo<T>(v));
      rawA[pidx<T>(j * NB + c)] = v;
    }
  } else {
    // lanes walk the tile's columns (contiguous p or q runs)
    const int64_t gcol = pp.s * pcol + q0 + ql;
    const bool ok = batch < pp.nbatch && q0 + ql < pp.s;  // ragged lane tiles
    int em = 1;
#pragma unroll 4
    for (int j = kg; j < R; j += Tf) {
      const Cx<H> v = ok ? load_elem<H, LOADOP, GROUP>(pp, in, batch, gcol + (int64_t)j * ms) : mk<H>(0, 0);
      if constexpr (kFx<T>) em = max(em, hexpo<T>(v));
      rawA[pidx<T>(j * NB + b)] = v;
    }
    if constexpr (kFx<T>) {
      if (active) atomicMax(colE + b, em);
    }
  }
  __syncthreads();

  // ---- the pass's R-point DFTs: radix sub-stages between the buffers
  const Cx<T>* twR = reinterpret_cast<const Cx<T>*>(pp.twR);
  const int cinb = kFx<T> ? 53 - B + colE[b] : 0;  // this thread's column, first sub-stage
  Cx<T>* cur = bufA;
  Cx<T>* nxt = bufB;
  bool raw = kFx<T>;  // cur holds unconverted FP64 values
#pragma unroll 1
  for (int si = 0; si < pp.nsub; ++si) {
    const SubStage& ss = pp.sub[si];
    const int sh = kFx<T> && si + 1 < pp.nsub ? fx_l(pp.sub[si + 1].r) : 0;
    bool moved = true;
    switch (ss.r) {
      case 2: substage_pp<T, DIR, 2>(cur, nxt, b, kg, Tf, NB, ss.Rr, ss.S, ss.fS, twR, sh, raw, cinb); break;
      case 3: substage_pp<T, DIR, 3>(cur, nxt, b, kg, Tf, NB, ss.Rr, ss.S, ss.fS, twR, sh, raw, cinb); break;
      case 4: substage_pp<T, DIR, 4>(cur, nxt, b, kg, Tf, NB, ss.Rr, ss.S, ss.fS, twR, sh, raw, cinb); break;
      case 5: substage_pp<T, DIR, 5>(cur, nxt, b, kg, Tf, NB, ss.Rr, ss.S, ss.fS, twR, sh, raw, cinb); break;
      case 7: substage_pp<T, DIR, 7>(cur, nxt, b, kg, Tf, NB, ss.Rr, ss.S, ss.fS, twR, sh, raw, cinb); break;
      case 8: substage_pp<T, DIR, 8>(cur, nxt, b, kg, Tf, NB, ss.Rr, ss.S, ss.fS, twR, sh, raw, cinb); break;
      case 11: substage_pp<T, DIR, 11>(cur, nxt, b, kg, Tf, NB, ss.Rr, ss.S, ss.fS, twR, sh, raw, cinb); break;
      case 13: substage_pp<T, DIR, 13>(cur, nxt, b, kg, Tf, NB, ss.Rr, ss.S, ss.fS, twR, sh, raw, cinb); break;
      case 16:
        if constexpr (sizeof(T) == 4) {
          if (pp.tc && tc16_fits(nthr, NB, ss.Rr)) {
            // tensor-core sub-stage: in place on the current buffer
            if (pp.tc == 1)
              substage_tc16<DIR, 1>(cur, tid, nthr, NB, ss.Rr, ss.S, ss.fS, pp.fNB, twR);
            else
              substage_tc16<DIR, 2>(cur, tid, nthr, NB, ss.Rr, ss.S, ss.fS, pp.fNB, twR);
            moved = false;
            break;
          }
        }
        substage_pp<T, DIR, 16>(cur, nxt, b, kg, Tf, NB, ss.Rr, ss.S, ss.fS, twR, sh, raw, cinb);
        break;
      default: break;
    }
    __syncthreads();
    raw = false;
    if (moved) {
      Cx<T>* t = cur;
      cur = nxt;
      nxt = t;
    }
  }

  // ---- store: shared -> HBM with the outer twiddle w_ncur^(p*j) and scale
  const OutConv<T> oc(pp);
  const bool tw = pp.tw_mode != 0;
  const Cx<H>* const rawc = reinterpret_cast<const Cx<H>*>(cur);
  // element at a padded position of column col (a pass without sub-stages
  // still holds the raw Fx inputs)
  auto elem = [&](int idx, int col) -> Cx<T> {
    if constexpr (kFx<T>) {
      if (raw) return to_c<T>(rawc[idx], 53 - B + colE[col]);
    }
    return cur[idx];
  };
  if (pp.store_rows) {
    // outputs contiguous along j (s == 1): lanes walk j
#pragma unroll 4
    for (int e = tid; e < E; e += nthr) {
      const int c = (int)pp.fR.div((uint32_t)e);
      const int j = e - c * R;
      const int cbt2 = (int)pp.fP.div((uint32_t)c);
      const int64_t bb = b0 + cbt2;
      if (bb < pp.nbatch) {
        const int64_t p = p0 + (c - cbt2 * P);
        Cx<T> v = elem(pidx<T>(j * NB + c), c);
        if (tw && p * j != 0) v = cmul(v, outer_tw<T>(pp, p * (int64_t)j));
        out[bb * pp.out_bstride + (int64_t)R * p + j] = oc(v, kFx<T> ? colE[c] : 0);
      }
    }
  } else {
    const bool ok = batch < pp.nbatch && q0 + ql < pp.s;
    if (ok) {
      Cx<H>* ob = out + batch * pp.out_bstride + (int64_t)R * pp.s * pcol + q0 + ql;
      const int Eb = kFx<T> ? colE[b] : 0;
#pragma unroll 4
      for (int j = kg; j < R; j += Tf) {
        Cx<T> v = elem(pidx<T>(j * NB + b), b);
        if (tw && pcol * j != 0) v = cmul(v, outer_tw<T>(pp, pcol * (int64_t)j));
        ob[(int64_t)j * pp.s] = oc(v, Eb);
      }
    }
  }
}

template <typename T, int DIR, int LOADOP, class Rec>
__device__ __forceinline__ void pass_body(const PassParams& pp, const void* __restrict__ in,
                                          Cx<Hs<T>>* __restrict__ out) {
  pass_tile<T, DIR, LOADOP, Rec, false>(pp, in, out, blockIdx.x, threadIdx.x, blockDim.x);
}

// load_elem with the batch offset already applied (boff = batch * stride)
template <typename T, int LOADOP>
__device__ __forceinline__ Cx<T> load_elem_off(const PassParams& pp, const void* in, int64_t boff, int64_t g) {
  if (LOADOP == LOAD_PLAIN) {
    return __ldg(reinterpret_cast<const Cx<T>*>(in) + boff + g);
  } else if (LOADOP == LOAD_DECONV) {
    const int64_t n = pp.ld_n, m = pp.ld_m, hp = pp.ld_hp, inner = pp.ld_inner > 1 ? pp.ld_inner : 1;
    int64_t a = g, i = 0;
    if (inner > 1) { a = g / inner; i = g - a * inner; }
    int64_t j;
    if (a < hp) j = a;
    else if (a >= m - n + hp) j = a - (m - n);
    else return mk<T>(0, 0);
    const Cx<T> x = __ldg(reinterpret_cast<const Cx<T>*>(in) + boff + j * inner + i);
    const T c = __ldg(reinterpret_cast<const T*>(pp.ld_tab) + j);
    return mk<T>(x.x * c, x.y * c);
  } else if (LOADOP == LOAD_SPREAD) {
    const int64_t n = pp.ld_n, inner = pp.ld_inner > 1 ? pp.ld_inner : 1;
    int64_t a = g, i = 0;
    if (inner > 1) { a = g / inner; i = g - a * inner; }
    const int w = pp.ld_w;
    const Cx<T>* x = reinterpret_cast<const Cx<T>*>(in) + boff + i;
    const T* wt = reinterpret_cast<const T*>(pp.ld_tab) + a * w;
    int64_t r = __ldg(pp.ld_l0 + a);
    T re = 0, im = 0;
    for (int o = 0; o < w; ++o) {
      const T c = __ldg(wt + o);
      const Cx<T> v = __ldg(x + r * inner);
      re = fma(c, v.x, re);
      im = fma(c, v.y, im);
      if (++r == n) r = 0;
    }
    return mk<T>(re, im);
  } else if (LOADOP == LOAD_C2R_PRE) {
    const int64_t h = pp.ld_n;
    const Cx<T>* X = reinterpret_cast<const Cx<T>*>(in) + boff;
    const Cx<T> a = __ldg(X + g);
    Cx<T> bb = __ldg(X + (h - g));
    bb.y = -bb.y;
    const T pre = half_or_one<T>(pp.ld_pre);  // 1/2 (irfft) or 1 (brfft)
    const Cx<T> xe = mk<T>((a.x + bb.x) * pre, (a.y + bb.y) * pre);
    const Cx<T> xd = mk<T>((a.x - bb.x) * pre, (a.y - bb.y) * pre);
    const Cx<T> w = c2r_twiddle<T>(pp, g);
    const T tr = fma(w.x, xd.x, -(w.y * xd.y));
    const T ti = fma(w.x, xd.y, w.y * xd.x);
    return mk<T>(xe.x - ti, xe.y + tr);
  } else {
    const T x = __ldg(reinterpret_cast<const T*>(in) + boff + g);
    return mk<T>(x, 0);
  }
}

// sub-stages 2 .. NS-DROP of a recipe (the first ran fused with the load;
// DROP = 1 leaves the last one to the fused store)
template <typename T, int DIR, int TF, int R, int S, int DROP, int NBC, int r, int... rest>
__device__ __forceinline__ void run_mid_skip(Cx<T>* buf, const int b, const int kg, const int NB,
                                             const Cx<T>* twR) {
  if constexpr (sizeof...(rest) >= DROP) {
    if constexpr (sizeof...(rest) == 0) {
      substage_ct<T, DIR, r, S, R / r, TF, NBC>(buf, b, kg, NB, twR);
    } else {
      substage_ct<T, DIR, r, S, R / r, TF, NBC, next_shift<r, rest...>()>(buf, b, kg, NB, twR);
      run_mid_skip<T, DIR, TF, R, S * r, DROP, NBC, rest...>(buf, b, kg, NB, twR);
    }
  }
}
template <typename T, int DIR, int TF, int R, int S1, int DROP, int NBC, int r0, int... rest>
__device__ __forceinline__ void run_mid_ct(Cx<T>* buf, const int b, const int kg, const int NB,
                                           const Cx<T>* twR) {
  if constexpr (sizeof...(rest) > 0) run_mid_skip<T, DIR, TF, R, S1, DROP, NBC, rest...>(buf, b, kg, NB, twR);
}

// Fused last sub-stage (radix rL) + HBM store of one tile: MODE 0 is the row
// store of a single-pass transform, MODE 1 the row store of a first pass
// (s == 1), MODE 2 the strided store of a later pass. Shared by the one-tile-per-CTA recipe
// kernels and the pipelined tensor-copy kernel (pass_tma.cuh).
template <typename T, int DIR, int MODE, int NBC, int... Rs>
__device__ __forceinline__ void store_last(const PassParams& pp, Cx<Hs<T>>* __restrict__ out,
                                           const Cx<T>* __restrict__ buf, const int tid, const int nthr,
                                           const int kg, const int b, const int64_t b0, const int64_t p0,
                                           const int64_t q0, const int ql, const int64_t batch,
                                           const int64_t pcol, const bool colok, const int* colE = nullptr) {
  using Rec = Recipe<Rs...>;
  constexpr int R = Rec::R, TF = Rec::Tf, NS = Rec::n;
  constexpr int rad[] = {Rs...};
  constexpr int rL = rad[NS - 1];
  const int NB = NBC > 0 ? NBC : pp.NB;
  const OutConv<T> oc(pp);
  using H = Hs<T>;
  const bool tw = pp.tw_mode != 0;
  if constexpr (MODE == 0) {
    // ---- fused last sub-stage (radix rL) + row store: butterfly u = c S + k
    // with k fastest across lanes writes outputs k + jj S of row c, the
    // lanes of a warp at consecutive addresses for each jj (one pass over
    // whole transforms: no outer twiddle)
    (void)tw;
    constexpr int S = R / rL;
    const int nbf = NB * S;
    for (int u = tid; u < nbf; u += nthr) {
      const int c = u / S;
      const int k = u - c * S;
      if (b0 + c >= pp.nbatch) continue;
      Cx<T> v[rL];
      if constexpr (NBC > 0 && LayC<T, NBC>::exact(S)) {
        const int base = LayC<T, NBC>::row(k) + LayC<T, NBC>::col(c);
#pragma unroll
        for (int j = 0; j < rL; ++j) v[j] = buf[base + j * LayC<T, NBC>::step(S)];
      } else {
#pragma unroll
        for (int j = 0; j < rL; ++j) v[j] = buf[pidx<T>((k + j * S) * NB + c)];
      }
      Dft<T, DIR, rL>::run(v);
      Cx<H>* o = out + (b0 + c) * pp.out_bstride + k;
      const int Ec = kFx<T> ? colE[c] : 0;
#pragma unroll
      for (int j = 0; j < rL; ++j) o[j * S] = oc(v[j], Ec);
    }
  } else if constexpr (MODE == 1) {
    // ---- fused last sub-stage (radix rL) + row store (s == 1). Butterfly
    // u = c S + k takes k fastest across lanes, so for each output
    // j = k + jj S the lanes of a warp write consecutive addresses of column
    // c's output row. F32: the outer twiddle w^((p0 + c) j) advances along
    // jj by w^((p0 + c) S), one complex multiply per output instead of a
    // table lookup (at most rL - 1 <= 15 steps); F64 passes are FP64-pipe
    // bound and keep the lookups.
    static_assert(NS >= 2, "a first pass has at least two sub-stages");
    constexpr int S = R / rL;
    constexpr bool kRecur = sizeof(T) == 4;
    const int nbf = NB * S;
    if (b0 < pp.nbatch) {
      Cx<H>* orow = out + b0 * pp.out_bstride + (int64_t)R * p0;
      for (int u = tid; u < nbf; u += nthr) {
        const int c = u / S;
        const int k = u - c * S;
        Cx<T> v[rL];
        if constexpr (NBC > 0 && LayC<T, NBC>::exact(S)) {
          const int base = LayC<T, NBC>::row(k) + LayC<T, NBC>::col(c);
#pragma unroll
          for (int j = 0; j < rL; ++j) v[j] = buf[base + j * LayC<T, NBC>::step(S)];
        } else {
#pragma unroll
          for (int j = 0; j < rL; ++j) v[j] = buf[pidx<T>((k + j * S) * NB + c)];
        }
        Dft<T, DIR, rL>::run(v);
        const uint32_t pc = (uint32_t)(p0 + c);
        uint32_t e = pc * (uint32_t)k;
        const uint32_t estep = pc * (uint32_t)S;
        Cx<T> w = mk<T>(1, 0), wstep = mk<T>(1, 0);
        if (kRecur && tw) {
          if (e != 0) w = outer_tw<T>(pp, e);
          if (estep != 0) wstep = outer_tw<T>(pp, estep);
        }
        Cx<H>* o = orow + (int64_t)R * c + k;
        const int Ec = kFx<T> ? colE[c] : 0;
#pragma unroll
        for (int j = 0; j < rL; ++j) {
          Cx<T> x = v[j];
          if (kRecur) {
            if (tw) {
              x = cmul(x, w);
              w = cmul(w, wstep);
            }
          } else if (tw && e != 0) {
            x = cmul(x, outer_tw<T>(pp, e));
          }
          o[j * S] = oc(x, Ec);
          e += estep;
        }
      }
    }
  } else {
    // ---- fused last sub-stage (radix rL, L = rL, no inner twiddle) + store:
    // butterfly k (< S = R/rL) writes positions j*S + k of its column
    constexpr int S = R / rL;
    constexpr int IPT = (S + TF - 1) / TF;
    Cx<T> v[IPT][rL];
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      const int k = kg + i * TF;
      if ((i + 1) * TF <= S || k < S) {
        if constexpr (NBC > 0 && LayC<T, NBC>::exact(S)) {
          const int base = LayC<T, NBC>::row(k) + LayC<T, NBC>::col(b);
#pragma unroll
          for (int j = 0; j < rL; ++j) v[i][j] = buf[base + j * LayC<T, NBC>::step(S)];
        } else {
#pragma unroll
          for (int j = 0; j < rL; ++j) v[i][j] = buf[pidx<T>((k + j * S) * NB + b)];
        }
      }
    }
    if (colok) {
      Cx<H>* ob = out + batch * pp.out_bstride + (int64_t)R * pp.s * pcol + q0 + ql;
      const int Eb = kFx<T> ? colE[b] : 0;
      const int64_t jstep = (int64_t)S * pp.s;
      const uint32_t estep = (uint32_t)pcol * (uint32_t)S;
      // F32: along a butterfly's outputs the outer twiddle w^(pcol (k + j S))
      // advances by w^(pcol S), one complex multiply per output instead of a
      // table lookup (at most rL - 1 <= 15 steps of rounding). F64 passes are
      // FP64-pipe bound and keep the lookups.
      constexpr bool kRecur = sizeof(T) == 4;
      const Cx<T> wstep = (kRecur && tw && estep != 0) ? outer_tw<T>(pp, estep) : mk<T>(1, 0);
#pragma unroll
      for (int i = 0; i < IPT; ++i) {
        const int k = kg + i * TF;
        if ((i + 1) * TF <= S || k < S) {
          Dft<T, DIR, rL>::run(v[i]);
          Cx<H>* o = ob + (int64_t)k * pp.s;
          uint32_t e = (uint32_t)pcol * (uint32_t)k;
          Cx<T> w = (kRecur && tw && e != 0) ? outer_tw<T>(pp, e) : mk<T>(1, 0);
#pragma unroll
          for (int j = 0; j < rL; ++j) {
            Cx<T> x = v[i][j];
            if (kRecur) {
              if (tw) {
                x = cmul(x, w);
                w = cmul(w, wstep);
              }
            } else if (tw && e != 0) {
              x = cmul(x, outer_tw<T>(pp, e));
            }
            *o = oc(x, Eb);
            o += jstep;
            e += estep;
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Recipe pass with the first sub-stage fused into the HBM load and/or the last
// sub-stage fused into the HBM store. MODE 0: lanes walk j on both sides (one
// pass over whole contiguous transforms); MODE 1: fused load, row store (the
// first pass of a multi-pass transform, s == 1); MODE 2: fused load and store
// (later passes: lanes walk the contiguous q columns on both sides).
// No per-element 64-bit multiply or multiply-high: addresses and (column,
// row) counters advance by additions.
template <typename T, int DIR, int LOADOP, int MODE, int NBC, int... Rs>
__device__ __forceinline__ void pass_fused(const PassParams& pp, const void* __restrict__ in,
                                           Cx<Hs<T>>* __restrict__ out) {
  using H = Hs<T>;
  using Rec = Recipe<Rs...>;
  constexpr int R = Rec::R, TF = Rec::Tf, NS = Rec::n;
  constexpr int rad[] = {Rs...};
  constexpr int r0 = rad[0], rL = rad[NS - 1];
  constexpr int EPT = (R + TF - 1) / TF;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* buf = reinterpret_cast<Cx<T>*>(smem_raw);
  uint32_t tile = blockIdx.x;
  if constexpr (LOADOP == LOAD_C2R_PRE && MODE == 1) {
    // The pre-pass reads X[g] and X[h - g]: entry g of tile tp is read again
    // as the mirror of tile tiles_p - 1 - tp (one column over). Launch order
    // interleaves each tile with its mirror (0, n-1, 1, n-2, ...), so both
    // reads of an entry are in flight together and the second hits L2.
    // tiles_q == 1 in a first pass.
    const uint32_t n = pp.tiles_p;
    const uint32_t bt = pp.ftp.div(tile);
    const uint32_t tl = tile - bt * n;
    tile = bt * n + ((tl & 1) ? n - 1 - (tl >> 1) : (tl >> 1));
  }
  const uint32_t t1 = pp.ftq.div(tile);
  const uint32_t tq = tile - t1 * pp.tiles_q;
  const uint32_t tb = pp.ftp.div(t1);
  const uint32_t tp = t1 - tb * pp.tiles_p;
  const int64_t q0 = (int64_t)tq * pp.Q, p0 = (int64_t)tp * pp.P, b0 = (int64_t)tb * pp.NBt;
  const int P = pp.P, Q = pp.Q, NB = NBC > 0 ? NBC : pp.NB;
  const int E = NB * R;
  const int tid = threadIdx.x, nthr = NBC > 0 ? NBC * TF : (int)blockDim.x;
  const int kg = NBC > 0 ? tid / NBC : (int)pp.fNB.div((uint32_t)tid);
  const int b = tid - kg * NB;
  const int cq = (int)pp.fQ.div((uint32_t)b);
  const int ql = b - cq * Q;
  const int cbt = (int)pp.fP.div((uint32_t)cq);
  const int pl = cq - cbt * P;
  const int64_t batch = b0 + cbt;
  const int64_t pcol = p0 + pl;
  const bool colok = batch < pp.nbatch && q0 + ql < pp.s;  // ragged lane tiles
  // the pass's inner twiddles w_R^t are staged in shared memory right after
  // the tile (smem_elems), so sub-stages read them with 32-bit shared
  // addresses: no per-element global index arithmetic
  // (large tables -- R beyond the planner's staging limit -- are read from
  // global memory instead, where they stay L1/L2-resident: staging them
  // would copy as many bytes per tile as the tile's data)
  const Cx<T>* twR = reinterpret_cast<const Cx<T>*>(pp.twR);
  if (pp.smem_tw_elems >= R) {
    Cx<T>* twS = buf + pp.smem_elems;
    const Cx<T>* twG = twR + tid;
    for (int t = tid; t < R; t += nthr, twG += nthr) twS[t] = ldt<T>(twG);
    twR = twS;
  }
  // Fx: exponent maximum of each tile column (after the tile and the staged
  // twiddles); made visible by the first barrier below
  int* const colE = reinterpret_cast<int*>(buf + pp.smem_elems + pp.smem_tw_elems);
  const int B = pp.fx_b0;
  constexpr int SH1 = next_shift<Rs...>();  // shift after the first sub-stage
  if constexpr (kFx<T>) {
    if (tid < NB) colE[tid] = 1;
  }

  if constexpr (MODE == 0 && NS >= 2) {
    // ---- fused row load + first sub-stage (radix r0, S = 1). Butterfly
    // u = c Rr + k takes k fastest across lanes: its inputs k + j Rr of row
    // c are read straight from HBM, consecutive lanes at consecutive
    // addresses for each j.
    constexpr int Rr = R / r0;
    const int nbf = NB * Rr;
    const int64_t bstr = LOADOP == LOAD_PLAIN ? pp.in_bstride : pp.ld_stride;
    __syncthreads();  // staged twiddles visible
    if constexpr (kFx<T>) {
      // column exponents first (the loop below loads the same elements
      // again, from L1/L2)
      for (int u = tid; u < nbf; u += nthr) {
        const int c = u / Rr;
        const int k = u - c * Rr;
        const int64_t bb = b0 + c;
        int em = 1;
        if (bb < pp.nbatch) {
#pragma unroll
          for (int j = 0; j < r0; ++j) em = max(em, hexpo<T>(load_elem_off<H, LOADOP>(pp, in, bb * bstr, k + j * Rr)));
        }
        col_expo_max(colE, c, em);
      }
      __syncthreads();
    }
    for (int u = tid; u < nbf; u += nthr) {
      const int c = u / Rr;
      const int k = u - c * Rr;
      const int64_t bb = b0 + c;
      const int cin = kFx<T> ? 53 - B + colE[c] : 0;
      Cx<T> v[r0];
      if (bb < pp.nbatch) {
#pragma unroll
        for (int j = 0; j < r0; ++j) v[j] = to_c<T>(load_elem_off<H, LOADOP>(pp, in, bb * bstr, k + j * Rr), cin);
      } else {
#pragma unroll
        for (int j = 0; j < r0; ++j) v[j] = mk<T>(0, 0);
      }
      Dft<T, DIR, r0>::run(v);
      const int a = r0 * k * NB + c;
      buf[pidx<T>(a)] = shr_c<T>(v[0], SH1);
#pragma unroll
      for (int j = 1; j < r0; ++j) {
        Cx<T> w = v[j];
        if (k != 0) w = cmul(w, twR[j * k]);
        buf[pidx<T>(a + j * NB)] = shr_c<T>(w, SH1);
      }
    }
    __syncthreads();
    if constexpr (NS > 2) {
      // middle sub-stages (the last one is fused into the row store)
      run_mid_ct<T, DIR, TF, R, r0, 1, NBC, Rs...>(buf, b, kg, NB, twR);
    }
  } else if constexpr (MODE == 0) {
    // ---- row load (lanes walk j): e = tid + i*nthr -> (c, j), c = column
    Cx<H> v[EPT];
    const int dc = nthr / R, dj = nthr - (nthr / R) * R;
    {
      int c = tid / R, j = tid - (tid / R) * R;
      const int64_t bstr = LOADOP == LOAD_PLAIN ? pp.in_bstride : pp.ld_stride;
      int64_t boff = (b0 + c) * bstr;
      const int64_t dstep = (int64_t)dc * bstr;
#pragma unroll
      for (int i = 0; i < EPT; ++i) {
        if (tid + i * nthr < E) {
          v[i] = b0 + c < pp.nbatch ? load_elem_off<H, LOADOP>(pp, in, boff, j) : mk<H>(0, 0);
        }
        j += dj; c += dc; boff += dstep;
        if (j >= R) { j -= R; c++; boff += bstr; }
      }
    }
    if constexpr (kFx<T>) {
      __syncthreads();  // column exponent initialisation visible
      int c = tid / R, j = tid - (tid / R) * R;
#pragma unroll
      for (int i = 0; i < EPT; ++i) {
        if (tid + i * nthr < E) col_expo_max(colE, c, hexpo<T>(v[i]));
        j += dj; c += dc;
        if (j >= R) { j -= R; c++; }
      }
      __syncthreads();
    }
    {
      int c = tid / R, j = tid - (tid / R) * R;
#pragma unroll
      for (int i = 0; i < EPT; ++i) {
        if (tid + i * nthr < E) buf[pidx<T>(j * NB + c)] = to_c<T>(v[i], kFx<T> ? 53 - B + colE[c] : 0);
        j += dj; c += dc;
        if (j >= R) { j -= R; c++; }
      }
    }
    __syncthreads();
    run_subs_ct<T, DIR, TF, R, 1, NBC, Rs...>(buf, b, kg, NB, twR);
  } else {
    // ---- fused load + first sub-stage (radix r0, S = 1): butterfly k reads
    // column positions k + j*R/r0 straight from HBM
    constexpr int Rr = R / r0;
    constexpr int IPT = (Rr + TF - 1) / TF;
    const int64_t ms = pp.m * pp.s;
    const int64_t bstr = LOADOP == LOAD_PLAIN ? pp.in_bstride : pp.ld_stride;
    const int64_t boff = batch * bstr;
    const int64_t gcol = pp.s * pcol + q0 + ql;
    Cx<H> h[IPT][r0];
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      const int k = kg + i * TF;
      if ((i + 1) * TF <= Rr || k < Rr) {
        int64_t g = gcol + (int64_t)k * ms;
        const int64_t gstep = (int64_t)Rr * ms;
        if constexpr (LOADOP == LOAD_C2R_PRE && MODE == 1) {
          if (pp.ld_tab3) {
            // entries g = pcol + (k + j Rr) m of the first pass: every
            // load of the butterfly first (both halves of each pair), then
            // the twiddle w_n^g = w_n^pcol w_2R^(k + j Rr) from the
            // thread's column factor and an R-entry table (L1-resident)
            // instead of two table reads per entry
            const int64_t hl = pp.ld_n;
            const Cx<H>* X = reinterpret_cast<const Cx<H>*>(in) + boff;
            const Cx<H>* tR = reinterpret_cast<const Cx<H>*>(pp.ld_tab3);
            Cx<H> xa[r0], xb[r0];
#pragma unroll
            for (int j = 0; j < r0; ++j) {
              const int64_t gj = g + j * gstep;
              xa[j] = colok ? __ldg(X + gj) : mk<H>(0, 0);
              xb[j] = colok ? __ldg(X + (hl - gj)) : mk<H>(0, 0);
            }
            const Cx<H> wp = colok ? c2r_twiddle<H>(pp, pcol) : mk<H>(1, 0);
            const H pre = half_or_one<H>(pp.ld_pre);
#pragma unroll
            for (int j = 0; j < r0; ++j) {
              const Cx<H> w = cmul(wp, __ldg(tR + k + j * Rr));
              h[i][j] = c2r_pre_combine<H>(xa[j], xb[j], w, pre);
            }
            continue;
          }
        }
#pragma unroll
        for (int j = 0; j < r0; ++j) {
          h[i][j] = colok ? load_elem_off<H, LOADOP>(pp, in, boff, g) : mk<H>(0, 0);
          g += gstep;
        }
      }
    }
    __syncthreads();  // staged twiddles visible (the loads above stay in flight)
    int cin = 0;
    if constexpr (kFx<T>) {
      int em = 1;
#pragma unroll
      for (int i = 0; i < IPT; ++i) {
        const int k = kg + i * TF;
        if ((i + 1) * TF <= Rr || k < Rr) {
#pragma unroll
          for (int j = 0; j < r0; ++j) em = max(em, hexpo<T>(h[i][j]));
        }
      }
      atomicMax(colE + b, em);
      __syncthreads();
      cin = 53 - B + colE[b];
    }
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      const int k = kg + i * TF;
      if ((i + 1) * TF <= Rr || k < Rr) {
        Cx<T> v[r0];
#pragma unroll
        for (int j = 0; j < r0; ++j) v[j] = to_c<T>(h[i][j], cin);
        Dft<T, DIR, r0>::run(v);
        const int a = r0 * k * NB + b;
        // compile-time columns: output rows r0 k + j are constant offsets
        // from row r0 k (a multiple of the rows per padding period)
        constexpr bool kLay = NBC > 0 && LayC<T, NBC>::exact(r0);
        const int base = kLay ? LayC<T, NBC>::row(r0 * k) + LayC<T, NBC>::col(b) : pidx<T>(a);
        buf[base] = shr_c<T>(v[0], SH1);
#pragma unroll
        for (int j = 1; j < r0; ++j) {
          Cx<T> w = v[j];
          if (NS > 1 && k != 0) w = cmul(w, twR[j * k]);
          buf[kLay ? base + LayC<T, NBC>::step(j) : pidx<T>(a + j * NB)] = shr_c<T>(w, SH1);
        }
      }
    }
    __syncthreads();
    if constexpr (NS > 2) {
      // middle sub-stages (the last one is fused into the store)
      run_mid_ct<T, DIR, TF, R, r0, 1, NBC, Rs...>(buf, b, kg, NB, twR);
    }
  }

  if constexpr (MODE == 1 || MODE == 2) {
    store_last<T, DIR, MODE, NBC, Rs...>(pp, out, buf, tid, nthr, kg, b, b0, p0, q0, ql, batch, pcol, colok, colE);
    return;
  }
  const OutConv<T> oc(pp);
  const bool tw = pp.tw_mode != 0;
  if constexpr (MODE == 0 && NS >= 2) {
    store_last<T, DIR, MODE, NBC, Rs...>(pp, out, buf, tid, nthr, kg, b, b0, p0, q0, ql, batch, pcol, colok, colE);
  } else if constexpr (MODE == 0) {
    // ---- row store (lanes walk j): outputs contiguous along j (s == 1)
    const int dc = nthr / R, dj = nthr - (nthr / R) * R;
    int c = tid / R, j = tid - (tid / R) * R;
    Cx<T> w[EPT];
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      w[i] = mk<T>(1, 0);
      if (tid + i * nthr < E && tw) {
        const uint32_t e = (uint32_t)(p0 + c) * (uint32_t)j;  // NBt == 1 whenever m > 1
        if (e != 0) w[i] = outer_tw<T>(pp, e);
      }
      j += dj; c += dc;
      if (j >= R) { j -= R; c++; }
    }
    c = tid / R; j = tid - (tid / R) * R;
    Cx<H>* op = out + b0 * pp.out_bstride + (int64_t)R * p0 + tid;
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const int e = tid + i * nthr;
      // column c is a batch entry
      if (e < E && b0 + c < pp.nbatch) {
        Cx<T> v = buf[pidx<T>(j * NB + c)];
        if (tw) v = cmul(v, w[i]);
        *op = oc(v, kFx<T> ? colE[c] : 0);
      }
      op += nthr;
      j += dj; c += dc;
      if (j >= R) { j -= R; c++; }
    }
  }
}

template <typename T, int DIR, int LOADOP, int MODE, int NBC, class Rec>
struct FusedLaunch;
template <typename T, int DIR, int LOADOP, int MODE, int NBC, int... Rs>
struct FusedLaunch<T, DIR, LOADOP, MODE, NBC, Recipe<Rs...>> {
  __device__ __forceinline__ static void run(const PassParams& pp, const void* in, Cx<Hs<T>>* out) {
    pass_fused<T, DIR, LOADOP, MODE, NBC, Rs...>(pp, in, out);
  }
};

}  // namespace fftj
