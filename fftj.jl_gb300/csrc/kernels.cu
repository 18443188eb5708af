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

#include "pass_common.cuh"

namespace fftj {

template <typename T, int DIR, int LOADOP>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256, 2)
    k_pass(const __grid_constant__ PassParams pp, const void* __restrict__ in, Cx<T>* __restrict__ out) {
  pass_body<T, DIR, LOADOP, RuntimeRecipe>(pp, in, out);
}

// Resampling interpolation (FFTJ _interp!, src/resample.jl:392-424; along a
// strided N-d axis, _rows_interp!, src/resample.jl:557-588): output (b, k, i)
// = sum_t wt[k*w + t] * grid(b, (l0[k] + t) mod m, i), i the inner index
// (fastest, so neighbouring threads read neighbouring grid elements).
template <typename T>
__global__ void k_interp(const __grid_constant__ InterpParams ip, const Cx<T>* __restrict__ g,
                         Cx<T>* __restrict__ y) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
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
    const Cx<T> gv = __ldg(gb + l * inner);
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
template <typename T, int B>
__global__ void k_hvdh_solve(const __grid_constant__ SolveParams sp, const Cx<T>* __restrict__ g,
                             Cx<T>* __restrict__ y) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
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
    if (__ldg(oi + i) >= 0) z = __ldg(gb + q);
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
    if (i < sp.H + sp.L && o >= 0) yb[o] = mk<T>(x.x * sc, x.y * sc);
  }
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
  } else if (cp.mode == 3) {  // complex copy of the first n entries
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] =
        reinterpret_cast<const Cx<T>*>(in)[b * cp.in_bstride + j];
  } else {  // irfft pre-pass (FFTJ src/real.jl:149-192) for a resampled inner transform
    const Cx<T>* X = reinterpret_cast<const Cx<T>*>(in) + b * cp.in_bstride;
    const int64_t h = cp.n;
    const Cx<T> a = X[j];
    Cx<T> bb = X[h - j];
    bb.y = -bb.y;
    const T pre = (T)cp.pre;
    const T xer = (a.x + bb.x) * pre, xei = (a.y + bb.y) * pre;
    const T xdr = (a.x - bb.x) * pre, xdi = (a.y - bb.y) * pre;
    const Cx<T> w = reinterpret_cast<const Cx<T>*>(cp.tab)[j];
    const T tr = fma(w.x, xdr, -(w.y * xdi));
    const T ti = fma(w.x, xdi, w.y * xdr);
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] = mk<T>(xer - ti, xei + tr);
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
      case LOAD_SPREAD: return k_pass<T, -1, LOAD_SPREAD>;
      default: return k_pass<T, -1, LOAD_PLAIN>;
    }
  }
  switch (load_op) {
    case LOAD_DECONV: return k_pass<T, 1, LOAD_DECONV>;
    case LOAD_C2R_PRE: return k_pass<T, 1, LOAD_C2R_PRE>;
    case LOAD_REAL: return k_pass<T, 1, LOAD_REAL>;
    case LOAD_SPREAD: return k_pass<T, 1, LOAD_SPREAD>;
    default: return k_pass<T, 1, LOAD_PLAIN>;
  }
}

// Opt a pass kernel into the device's largest dynamic shared memory. The
// attribute belongs to the kernel function (shared by every plan), so it is
// never set below the maximum any plan may need.
template <typename T>
cudaError_t prepare_pass(const PassParams& pp, int dir, const void* fn) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const size_t need = (size_t)(pp.smem_elems + pp.smem_tw_elems) * sizeof(Cx<T>);
  if (need > (size_t)optin) return cudaErrorInvalidValue;
  const void* f = fn ? fn : (const void*)pass_fn<T>(dir, pp.load_op);
  return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

template <typename T>
cudaError_t launch_pass(const PassParams& pp, int dir, const void* fn, const void* in, void* out,
                        cudaStream_t st) {
  const size_t smem = (size_t)(pp.smem_elems + pp.smem_tw_elems) * sizeof(Cx<T>);
  const uint32_t grid = pp.tiles_q * pp.tiles_p * pp.tiles_b;
  const void* f = fn ? fn : (const void*)pass_fn<T>(dir, pp.load_op);
  void* args[3] = {const_cast<PassParams*>(&pp), const_cast<void**>(&in), &out};
  return cudaLaunchKernel(f, dim3(grid), dim3(pp.threads), args, smem, st);
}

template <typename T>
cudaError_t launch_interp(const InterpParams& ip, const void* g, void* y, cudaStream_t st) {
  const int64_t total = ip.n * ip.nbatch * (ip.inner > 1 ? ip.inner : 1);
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

template <typename T>
cudaError_t launch_solve(const SolveParams& sp, const void* g, void* y, cudaStream_t st) {
  const int64_t total = sp.nbatch * sp.nchunk;
  const int th = 128;
  const unsigned grid = (unsigned)((total + th - 1) / th);
  auto gg = reinterpret_cast<const Cx<T>*>(g);
  auto yy = reinterpret_cast<Cx<T>*>(y);
  switch (sp.B) {
    case 1: k_hvdh_solve<T, 1><<<grid, th, 0, st>>>(sp, gg, yy); break;
    case 2: k_hvdh_solve<T, 2><<<grid, th, 0, st>>>(sp, gg, yy); break;
    case 3: k_hvdh_solve<T, 3><<<grid, th, 0, st>>>(sp, gg, yy); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template cudaError_t launch_solve<float>(const SolveParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_solve<double>(const SolveParams&, const void*, void*, cudaStream_t);
template cudaError_t prepare_pass<float>(const PassParams&, int, const void*);
template cudaError_t prepare_pass<double>(const PassParams&, int, const void*);
template cudaError_t launch_pass<float>(const PassParams&, int, const void*, const void*, void*, cudaStream_t);
template cudaError_t launch_pass<double>(const PassParams&, int, const void*, const void*, void*, cudaStream_t);
template cudaError_t launch_interp<float>(const InterpParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_interp<double>(const InterpParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_real_post<float>(const RealPostParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_real_post<double>(const RealPostParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_copy<float>(const CopyParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_copy<double>(const CopyParams&, const void*, void*, cudaStream_t);

}  // namespace fftj
