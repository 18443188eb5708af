// Elementwise ops of the transform path (interpolation, banded solve, real
// post-pass, copies), one output element (or solve chunk) per call, shared
// by their own kernels (kernels.cu) and the persistent group kernel
// (group.cu). CG selects L2-coherent data loads (group kernel).
#pragma once
#include <cuda_runtime.h>

#include "pass_common.cuh"

namespace fftj {

// Resampling interpolation (FFTJ _interp!, src/resample.jl:392-424; along a
// strided N-d axis, _rows_interp!, src/resample.jl:557-588): output (b, k, i)
// = sum_t wt[k*w + t] * grid(b, (l0[k] + t) mod m, i), i the inner index
// (fastest, so neighbouring threads read neighbouring grid elements).
template <typename T, bool CG>
__device__ __forceinline__ void interp_at(const InterpParams& ip, const Cx<T>* __restrict__ g,
                                          Cx<T>* __restrict__ y, const int64_t idx) {
  const int64_t inner = ip.inner > 1 ? ip.inner : 1;
  if (idx >= ip.n * ip.nbatch * inner) return;
  int64_t rest = idx, i = 0;
  if (inner > 1) { rest = idx / inner; i = idx - rest * inner; }
  const int64_t b = rest / ip.n, k = rest - b * ip.n;
  const T* wt = reinterpret_cast<const T*>(ip.wt) + k * ip.w;
  const Cx<T>* gb = g + b * ip.g_bstride + i;
  int64_t l = __ldg(ip.l0 + k);
  if (l < 0) l += ip.m;
  T re = 0, im = 0;
  for (int t = 0; t < ip.w; ++t) {
    const T wv = __ldg(wt + t);
    const Cx<T> gv = ldd<CG>(gb + l * inner);
    re = fma(wv, gv.x, re);
    im = fma(wv, gv.y, im);
    ++l;
    if (l >= ip.m) l -= ip.m;
  }
  y[b * ip.y_bstride + k * inner + i] = mk<T>(re, im);
}

// HvdH banded solve (FFTJ _hvdh_subst! / _hvdh_back!, src/hvdh.jl:604-686):
// thread (b, c) runs forward substitution over its chunk's R rows (rows q0
// .. q0+R-1 of the length-t transform, cyclic), keeping z in a strided
// scratch, then back substitution, writing the core rows' unknowns to their
// permuted outputs, scaled by scale * n / t.
template <typename T, int B, bool CG>
__device__ __forceinline__ void solve_at(const SolveParams& sp, const Cx<T>* __restrict__ g,
                                         Cx<T>* __restrict__ y, const int64_t tid) {
  const int64_t nt = sp.nbatch * sp.nchunk;
  if (tid >= nt) return;
  const int64_t b = tid / sp.nchunk, ch = tid - b * sp.nchunk;
  const int64_t R = sp.R, t = sp.t;
  const T* lf = reinterpret_cast<const T*>(sp.lf) + ch * R * B;
  const T* uf = reinterpret_cast<const T*>(sp.uf) + ch * R * (B + 1);
  const int32_t* oi = sp.oi + ch * R;
  Cx<T>* zw = reinterpret_cast<Cx<T>*>(sp.zw) + tid;
  const Cx<T>* gb = g + b * sp.g_bstride;
  int64_t q = ch * sp.L - sp.H;
  q = ((q % t) + t) % t;
  Cx<T> zp[B];
#pragma unroll
  for (int k = 0; k < B; ++k) zp[k] = mk<T>(0, 0);  // zp[k] = z_{i-1-k}
  for (int64_t i = 0; i < R; ++i) {
    Cx<T> z = mk<T>(0, 0);
    if (__ldg(oi + i) >= 0) z = ldd<CG>(gb + q);
#pragma unroll
    for (int k = 0; k < B; ++k) {
      const T f = __ldg(lf + i * B + k);
      z.x = fma(-f, zp[k].x, z.x);
      z.y = fma(-f, zp[k].y, z.y);
    }
#pragma unroll
    for (int k = B - 1; k > 0; --k) zp[k] = zp[k - 1];
    zp[0] = z;
    zw[i * nt] = z;
    if (++q == t) q = 0;
  }
  Cx<T> xp[B];
#pragma unroll
  for (int k = 0; k < B; ++k) xp[k] = mk<T>(0, 0);  // xp[k] = x_{i+1+k}
  const T sc = (T)sp.sc;
  Cx<T>* yb = y + b * sp.y_bstride;
  for (int64_t i = R - 1; i >= sp.H; --i) {
    Cx<T> x = zw[i * nt];
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const T u = __ldg(uf + i * (B + 1) + 1 + j);
      x.x = fma(-u, xp[j].x, x.x);
      x.y = fma(-u, xp[j].y, x.y);
    }
    const T iu = __ldg(uf + i * (B + 1));
    x.x *= iu;
    x.y *= iu;
#pragma unroll
    for (int k = B - 1; k > 0; --k) xp[k] = xp[k - 1];
    xp[0] = x;
    const int32_t o = __ldg(oi + i);
    if (i < sp.H + sp.L && o >= 0) {
      Cx<T> v = mk<T>(x.x * sc, x.y * sc);
      if (sp.tw) v = cmul(v, __ldg(reinterpret_cast<const Cx<T>*>(sp.tw) + (b % sp.tw_s) * (int64_t)o));
      yb[o] = v;
    }
  }
}

// rfft even post-pass (FFTJ src/real.jl:85-135): X[k] = xe + w (-i xo).
template <typename T, bool CG>
__device__ __forceinline__ void real_post_at(const RealPostParams& rp, const Cx<T>* __restrict__ z,
                                             Cx<T>* __restrict__ y, const int64_t idx) {
  const int64_t h = rp.h;
  if (idx >= (h + 1) * rp.nbatch) return;
  const int64_t b = idx / (h + 1), k = idx - b * (h + 1);
  const Cx<T>* Z = z + b * rp.z_bstride;
  Cx<T> out;
  if (k == 0 || k == h) {
    const Cx<T> z0 = ldd<CG>(Z);
    out = mk<T>(k == 0 ? z0.x + z0.y : z0.x - z0.y, 0);
  } else {
    const Cx<T> a = ldd<CG>(Z + k);
    Cx<T> bb = ldd<CG>(Z + (h - k));
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
template <typename T, bool CG>
__device__ __forceinline__ void copy_at(const CopyParams& cp, const void* __restrict__ in, void* __restrict__ out,
                                        const int64_t idx) {
  if (idx >= cp.n * cp.nbatch) return;
  const int64_t b = idx / cp.n, j = idx - b * cp.n;
  if (cp.mode == 0) {  // real -> complex
    const T x = ldd<CG>(reinterpret_cast<const T*>(in) + b * cp.in_bstride + j);
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] = mk<T>(x, 0);
  } else if (cp.mode == 1) {  // hermitian expansion of nc = n/2+1 values to n
    const Cx<T>* X = reinterpret_cast<const Cx<T>*>(in) + b * cp.in_bstride;
    Cx<T> v;
    if (j < cp.nc) v = ldd<CG>(X + j);
    else { v = ldd<CG>(X + (cp.n - j)); v.y = -v.y; }
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] = v;
  } else if (cp.mode == 2) {  // complex -> real part
    const Cx<T> v = ldd<CG>(reinterpret_cast<const Cx<T>*>(in) + b * cp.in_bstride + j);
    reinterpret_cast<T*>(out)[b * cp.out_bstride + j] = v.x;
  } else if (cp.mode == 3) {  // complex copy of the first n entries
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] =
        ldd<CG>(reinterpret_cast<const Cx<T>*>(in) + b * cp.in_bstride + j);
  } else if (cp.mode == 5) {  // decimation in time (FFTJ _split_gather!, src/composite.jl:245-252)
    const int64_t sd = cp.nc, pl = cp.n / sd;
    const int64_t r = j / pl, jj = j - r * pl;
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] =
        ldd<CG>(reinterpret_cast<const Cx<T>*>(in) + b * cp.in_bstride + r + sd * jj);
  } else {  // irfft pre-pass (FFTJ src/real.jl:149-192) for a resampled inner transform
    const Cx<T>* X = reinterpret_cast<const Cx<T>*>(in) + b * cp.in_bstride;
    const int64_t h = cp.n;
    const Cx<T> a = ldd<CG>(X + j);
    Cx<T> bb = ldd<CG>(X + (h - j));
    bb.y = -bb.y;
    const T pre = half_or_one<T>(cp.pre);  // 1/2 (irfft) or 1 (brfft)
    const T xer = (a.x + bb.x) * pre, xei = (a.y + bb.y) * pre;
    const T xdr = (a.x - bb.x) * pre, xdi = (a.y - bb.y) * pre;
    const Cx<T> w = reinterpret_cast<const Cx<T>*>(cp.tab)[j];
    const T tr = fma(w.x, xdr, -(w.y * xdi));
    const T ti = fma(w.x, xdi, w.y * xdr);
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] = mk<T>(xer - ti, xei + tr);
  }
}

}  // namespace fftj
