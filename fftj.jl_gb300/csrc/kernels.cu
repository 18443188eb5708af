// sm_103a kernels of the FFTJ transform path.
//
// The hot kernel is one Stockham "super-radix" pass (k_pass): each CTA loads a
// tile of butterfly columns (batch x p x q) from HBM with coalesced accesses,
// runs the pass's R-point DFTs as a chain of register radix sub-stages
// (2/3/4/5/7/8/11/13/16) ping-ponging through shared memory, applies the
// pass's outer twiddle w_ncur^(p*j) and writes the tile back. A 1-D transform
// of length N = R1*R2*...*Rk is k such passes (the Stockham stage of
// FFTJ's src/stockham.jl:26-130 with radix R_i instead of 4/8), i.e. the
// four-step/six-step family (src/fourstep.jl) with the transposes folded into
// the Stockham index maps. N-d passes are the same kernel with the inner
// dims folded into the stride s (src/ndplan.jl:1-5: "effective stride s*Bi").
#include <cuda_runtime.h>

#include "bfly_consts.h"
#include "fftj_internal.h"

namespace fftj {

template <typename T>
struct CT;
template <>
struct CT<float> { using t = float2; };
template <>
struct CT<double> { using t = double2; };

template <typename T>
using Cx = typename CT<T>::t;

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
// One radix-r Stockham sub-stage on all NB columns of the tile, in place:
// element j of sub-butterfly k (= p*S + q) is read at position k + j*R/r and
// written at r*S*p + j*S + q, twiddled by w_L^(p*j) = w_R^(p*j*S). Every
// thread first loads all of its (at most max(1, 16/r)) butterflies into
// registers, so one shared buffer suffices; the host sizes the CTA so that
// every sub-stage's butterflies fit (threads * IPT(r) >= tile / r).
template <typename T, int DIR, int r>
__device__ __noinline__ void substage(Cx<T>* __restrict__ buf, const int NB, const FastDiv fNB, const int Rr,
                                      const int S, const FastDiv fS, const Cx<T>* __restrict__ twR) {
  constexpr int IPT = (16 / r) > 0 ? (16 / r) : 1;
  const int items = NB * Rr;
  Cx<T> v[IPT][r];
#pragma unroll
  for (int i = 0; i < IPT; ++i) {
    const int it = threadIdx.x + i * blockDim.x;
    if (it < items) {
      const int k = (int)fNB.div((uint32_t)it);
      const int b = it - k * NB;
#pragma unroll
      for (int j = 0; j < r; ++j) v[i][j] = buf[pidx<T>((k + j * Rr) * NB + b)];
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < IPT; ++i) {
    const int it = threadIdx.x + i * blockDim.x;
    if (it < items) {
      const int k = (int)fNB.div((uint32_t)it);
      const int b = it - k * NB;
      const int p = (int)fS.div((uint32_t)k);
      const int q = k - p * S;
      Dft<T, DIR, r>::run(v[i]);
      const int ob = r * S * p + q;
      buf[pidx<T>(ob * NB + b)] = v[i][0];
      if (p == 0) {
#pragma unroll
        for (int j = 1; j < r; ++j) buf[pidx<T>((ob + j * S) * NB + b)] = v[i][j];
      } else {
#pragma unroll
        for (int j = 1; j < r; ++j) {
          const Cx<T> w = __ldg(&twR[p * j * S]);
          buf[pidx<T>((ob + j * S) * NB + b)] = cmul(v[i][j], w);
        }
      }
    }
  }
  __syncthreads();
}

template <typename T, int LOADOP>
__device__ __forceinline__ Cx<T> load_elem(const PassParams& pp, const void* in, int64_t b, int64_t g) {
  if (LOADOP == LOAD_PLAIN) {
    return __ldg(reinterpret_cast<const Cx<T>*>(in) + b * pp.in_bstride + g);
  } else if (LOADOP == LOAD_DECONV) {
    // grid position g of the length-m zero-padded deconvolved input
    // (FFTJ _deconv! + zero fill, src/resample.jl:258-301)
    const int64_t n = pp.ld_n, m = pp.ld_m, hp = pp.ld_hp;
    int64_t j;
    if (g < hp) j = g;
    else if (g >= m - n + hp) j = g - (m - n);
    else return mk<T>(0, 0);
    const Cx<T> x = __ldg(reinterpret_cast<const Cx<T>*>(in) + b * pp.ld_stride + j);
    const T c = __ldg(reinterpret_cast<const T*>(pp.ld_tab) + j);
    return mk<T>(x.x * c, x.y * c);
  } else if (LOADOP == LOAD_C2R_PRE) {
    // irfft pre-pass (FFTJ src/real.jl:149-192): Z[k] = xe + i (w xd)
    const int64_t h = pp.ld_n;
    const Cx<T>* X = reinterpret_cast<const Cx<T>*>(in) + b * pp.ld_stride;
    const Cx<T> a = __ldg(X + g);
    Cx<T> bb = __ldg(X + (h - g));
    bb.y = -bb.y;
    const T pre = (T)pp.ld_pre;
    const Cx<T> xe = mk<T>((a.x + bb.x) * pre, (a.y + bb.y) * pre);
    const Cx<T> xd = mk<T>((a.x - bb.x) * pre, (a.y - bb.y) * pre);
    const Cx<T> w = __ldg(reinterpret_cast<const Cx<T>*>(pp.ld_tab) + g);
    const T tr = fma(w.x, xd.x, -(w.y * xd.y));
    const T ti = fma(w.x, xd.y, w.y * xd.x);
    return mk<T>(xe.x - ti, xe.y + tr);
  } else {  // LOAD_REAL
    const T x = __ldg(reinterpret_cast<const T*>(in) + b * pp.ld_stride + g);
    return mk<T>(x, 0);
  }
}

template <typename T>
__device__ __forceinline__ Cx<T> outer_tw(const PassParams& pp, int64_t e) {
  if (pp.tw_mode == 1) return __ldg(reinterpret_cast<const Cx<T>*>(pp.tw_full) + e);
  const Cx<T> hi = __ldg(reinterpret_cast<const Cx<T>*>(pp.tw_hi) + (e >> pp.tw_shift));
  const Cx<T> lo = __ldg(reinterpret_cast<const Cx<T>*>(pp.tw_lo) + (e & ((1ll << pp.tw_shift) - 1)));
  return cmul(hi, lo);
}

template <typename T, int DIR, int LOADOP>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256, 2) k_pass(const __grid_constant__ PassParams pp, const void* __restrict__ in,
                                              Cx<T>* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx<T>* bufA = reinterpret_cast<Cx<T>*>(smem_raw);
  const uint32_t tile = blockIdx.x;
  const uint32_t t1 = pp.ftq.div(tile);
  const uint32_t tq = tile - t1 * pp.tiles_q;
  const uint32_t tb = pp.ftp.div(t1);
  const uint32_t tp = t1 - tb * pp.tiles_p;
  const int64_t q0 = (int64_t)tq * pp.Q, p0 = (int64_t)tp * pp.P, b0 = (int64_t)tb * pp.NBt;
  const int R = pp.R, P = pp.P, Q = pp.Q, NB = pp.NB;
  const int E = NB * R;
  const int64_t ms = pp.m * pp.s;

  // load: order (ql fastest, pl, j, bt) follows the input's contiguous runs.
  // Every thread owns at most 16 elements (threads >= tile / 16); all of its
  // global loads are issued before the first shared-memory store.
  constexpr int EPT = 16;
  {
    Cx<T> v[EPT];
    int sidx[EPT];
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const int e = threadIdx.x + i * blockDim.x;
      sidx[i] = -1;
      if (e < E) {
        const uint32_t t = pp.fQ.div((uint32_t)e);
        const int ql = e - (int)t * Q;
        const uint32_t t2 = pp.fP.div(t);
        const int pl = (int)t - (int)t2 * P;
        const uint32_t bt = pp.fR.div(t2);
        const int j = (int)t2 - (int)bt * R;
        const int64_t b = b0 + bt;
        v[i] = mk<T>(0, 0);
        if (b < pp.nbatch) {
          const int64_t g = pp.s * (p0 + pl) + (int64_t)j * ms + q0 + ql;
          v[i] = load_elem<T, LOADOP>(pp, in, b, g);
        }
        sidx[i] = pidx<T>(j * NB + ((int)bt * P + pl) * Q + ql);
      }
    }
#pragma unroll
    for (int i = 0; i < EPT; ++i)
      if (sidx[i] >= 0) bufA[sidx[i]] = v[i];
  }
  __syncthreads();

  const Cx<T>* twR = reinterpret_cast<const Cx<T>*>(pp.twR);
#pragma unroll 1
  for (int i = 0; i < pp.nsub; ++i) {
    const SubStage& ss = pp.sub[i];
    switch (ss.r) {
      case 2: substage<T, DIR, 2>(bufA, pp.NB, pp.fNB, ss.Rr, ss.S, ss.fS, twR); break;
      case 3: substage<T, DIR, 3>(bufA, pp.NB, pp.fNB, ss.Rr, ss.S, ss.fS, twR); break;
      case 4: substage<T, DIR, 4>(bufA, pp.NB, pp.fNB, ss.Rr, ss.S, ss.fS, twR); break;
      case 5: substage<T, DIR, 5>(bufA, pp.NB, pp.fNB, ss.Rr, ss.S, ss.fS, twR); break;
      case 7: substage<T, DIR, 7>(bufA, pp.NB, pp.fNB, ss.Rr, ss.S, ss.fS, twR); break;
      case 8: substage<T, DIR, 8>(bufA, pp.NB, pp.fNB, ss.Rr, ss.S, ss.fS, twR); break;
      case 11: substage<T, DIR, 11>(bufA, pp.NB, pp.fNB, ss.Rr, ss.S, ss.fS, twR); break;
      case 13: substage<T, DIR, 13>(bufA, pp.NB, pp.fNB, ss.Rr, ss.S, ss.fS, twR); break;
      case 16: substage<T, DIR, 16>(bufA, pp.NB, pp.fNB, ss.Rr, ss.S, ss.fS, twR); break;
      default: break;
    }
  }

  // store: order (ql fastest, j, pl, bt) follows the output's contiguous runs;
  // the outer twiddle loads of all of a thread's elements are issued together.
  const bool scaled = pp.scale != 1.0;
  const T sc = (T)pp.scale;
  Cx<T> v[EPT];
  int64_t gout[EPT];
#pragma unroll
  for (int i = 0; i < EPT; ++i) {
    const int e = threadIdx.x + i * blockDim.x;
    gout[i] = -1;
    if (e < E) {
      const uint32_t t = pp.fQ.div((uint32_t)e);
      const int ql = e - (int)t * Q;
      const uint32_t t2 = pp.fR.div(t);
      const int j = (int)t - (int)t2 * R;
      const uint32_t bt = pp.fP.div(t2);
      const int pl = (int)t2 - (int)bt * P;
      const int64_t b = b0 + bt;
      if (b < pp.nbatch) {
        const int col = ((int)bt * P + pl) * Q + ql;
        v[i] = bufA[pidx<T>(j * NB + col)];
        const int64_t p = p0 + pl;
        if (pp.tw_mode != 0 && p * j != 0) v[i] = cmul(v[i], outer_tw<T>(pp, p * (int64_t)j));
        gout[i] = b * pp.out_bstride + (int64_t)R * pp.s * p + (int64_t)j * pp.s + q0 + ql;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < EPT; ++i) {
    if (gout[i] >= 0) {
      Cx<T> w = v[i];
      if (scaled) { w.x *= sc; w.y *= sc; }
      out[gout[i]] = w;
    }
  }
}

// Resampling interpolation (FFTJ _interp!, src/resample.jl:392-424).
template <typename T>
__global__ void k_interp(const __grid_constant__ InterpParams ip, const Cx<T>* __restrict__ g, Cx<T>* __restrict__ y) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= ip.n * ip.nbatch) return;
  const int64_t b = idx / ip.n, k = idx - b * ip.n;
  const T* wt = reinterpret_cast<const T*>(ip.wt) + k * ip.w;
  const Cx<T>* gb = g + b * ip.g_bstride;
  int64_t l = __ldg(ip.l0 + k);
  if (l < 0) l += ip.m;
  T re = 0, im = 0;
  for (int i = 0; i < ip.w; ++i) {
    const T wv = __ldg(wt + i);
    const Cx<T> gv = __ldg(gb + l);
    re = fma(wv, gv.x, re);
    im = fma(wv, gv.y, im);
    ++l;
    if (l >= ip.m) l -= ip.m;
  }
  y[b * ip.y_bstride + k] = mk<T>(re, im);
}

// rfft even post-pass (FFTJ src/real.jl:85-135): X[k] = xe + w (-i xo).
template <typename T>
__global__ void k_real_post(const RealPostParams rp, const Cx<T>* __restrict__ z, Cx<T>* __restrict__ y) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t h = rp.h;
  if (idx >= (h + 1) * rp.nbatch) return;
  const int64_t b = idx / (h + 1), k = idx - b * (h + 1);
  const Cx<T>* Z = z + b * rp.z_bstride;
  Cx<T> out;
  if (k == 0 || k == h) {
    const Cx<T> z0 = __ldg(Z);
    out = mk<T>(k == 0 ? z0.x + z0.y : z0.x - z0.y, 0);
  } else {
    const Cx<T> a = __ldg(Z + k);
    Cx<T> bb = __ldg(Z + (h - k));
    bb.y = -bb.y;
    const T half = (T)0.5;
    const T xer = (a.x + bb.x) * half, xei = (a.y + bb.y) * half;
    const T xor_ = (a.x - bb.x) * half, xoi = (a.y - bb.y) * half;
    const Cx<T> w = __ldg(reinterpret_cast<const Cx<T>*>(rp.tw) + k);
    out = mk<T>(xer + fma(w.x, xoi, w.y * xor_), xei + fma(w.y, xoi, -(w.x * xor_)));
  }
  y[b * rp.y_bstride + k] = out;
}

// Odd-length real edges (FFTJ src/real.jl:136-140, 194-209).
template <typename T>
__global__ void k_copy(const CopyParams cp, const void* __restrict__ in, void* __restrict__ out) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= cp.n * cp.nbatch) return;
  const int64_t b = idx / cp.n, j = idx - b * cp.n;
  if (cp.mode == 0) {  // real -> complex
    const T x = reinterpret_cast<const T*>(in)[b * cp.in_bstride + j];
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] = mk<T>(x, 0);
  } else if (cp.mode == 1) {  // hermitian expansion of nc = n/2+1 values to n
    const Cx<T>* X = reinterpret_cast<const Cx<T>*>(in) + b * cp.in_bstride;
    Cx<T> v;
    if (j < cp.nc) v = X[j];
    else { v = X[cp.n - j]; v.y = -v.y; }
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] = v;
  } else if (cp.mode == 2) {  // complex -> real part
    const Cx<T> v = reinterpret_cast<const Cx<T>*>(in)[b * cp.in_bstride + j];
    reinterpret_cast<T*>(out)[b * cp.out_bstride + j] = v.x;
  } else {  // complex copy of the first n entries
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] =
        reinterpret_cast<const Cx<T>*>(in)[b * cp.in_bstride + j];
  }
}

// ---------------------------------------------------------------------------
template <typename T>
using PassFn = void (*)(const PassParams, const void*, Cx<T>*);

template <typename T>
static PassFn<T> pass_fn(int dir, int load_op) {
  if (dir < 0) {
    switch (load_op) {
      case LOAD_DECONV: return k_pass<T, -1, LOAD_DECONV>;
      case LOAD_C2R_PRE: return k_pass<T, -1, LOAD_C2R_PRE>;
      case LOAD_REAL: return k_pass<T, -1, LOAD_REAL>;
      default: return k_pass<T, -1, LOAD_PLAIN>;
    }
  }
  switch (load_op) {
    case LOAD_DECONV: return k_pass<T, 1, LOAD_DECONV>;
    case LOAD_C2R_PRE: return k_pass<T, 1, LOAD_C2R_PRE>;
    case LOAD_REAL: return k_pass<T, 1, LOAD_REAL>;
    default: return k_pass<T, 1, LOAD_PLAIN>;
  }
}

// Opt the pass kernel into the device's largest dynamic shared memory. The
// attribute belongs to the kernel function (shared by every plan), so it is
// never set below the maximum any plan may need.
template <typename T>
cudaError_t prepare_pass(const PassParams& pp, int dir) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const size_t need = (size_t)pp.smem_elems * sizeof(Cx<T>);
  if (need > (size_t)optin) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(pass_fn<T>(dir, pp.load_op), cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

template <typename T>
cudaError_t launch_pass(const PassParams& pp, int dir, const void* in, void* out, cudaStream_t st) {
  const size_t smem = (size_t)pp.smem_elems * sizeof(Cx<T>);
  const uint32_t grid = pp.tiles_q * pp.tiles_p * pp.tiles_b;
  pass_fn<T>(dir, pp.load_op)<<<grid, pp.threads, smem, st>>>(pp, in, reinterpret_cast<Cx<T>*>(out));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_interp(const InterpParams& ip, const void* g, void* y, cudaStream_t st) {
  const int64_t total = ip.n * ip.nbatch;
  const int th = 256;
  k_interp<T><<<(unsigned)((total + th - 1) / th), th, 0, st>>>(ip, reinterpret_cast<const Cx<T>*>(g),
                                                                reinterpret_cast<Cx<T>*>(y));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_real_post(const RealPostParams& rp, const void* z, void* y, cudaStream_t st) {
  const int64_t total = (rp.h + 1) * rp.nbatch;
  const int th = 256;
  k_real_post<T><<<(unsigned)((total + th - 1) / th), th, 0, st>>>(rp, reinterpret_cast<const Cx<T>*>(z),
                                                                   reinterpret_cast<Cx<T>*>(y));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_copy(const CopyParams& cp, const void* in, void* out, cudaStream_t st) {
  const int64_t total = cp.n * cp.nbatch;
  const int th = 256;
  k_copy<T><<<(unsigned)((total + th - 1) / th), th, 0, st>>>(cp, in, out);
  return cudaGetLastError();
}

template cudaError_t prepare_pass<float>(const PassParams&, int);
template cudaError_t prepare_pass<double>(const PassParams&, int);
template cudaError_t launch_pass<float>(const PassParams&, int, const void*, void*, cudaStream_t);
template cudaError_t launch_pass<double>(const PassParams&, int, const void*, void*, cudaStream_t);
template cudaError_t launch_interp<float>(const InterpParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_interp<double>(const InterpParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_real_post<float>(const RealPostParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_real_post<double>(const RealPostParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_copy<float>(const CopyParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_copy<double>(const CopyParams&, const void*, void*, cudaStream_t);

}  // namespace fftj
