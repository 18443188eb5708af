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

// Thread -> (sequence b, chunk ch, lane i) of a banded solve. Along a
// strided axis (HvPass lanes, sp.inner > 1: row r of lane i at r * inner +
// i) lanes are fastest, so a warp's grid reads and output writes are
// adjacent and its factor reads are one broadcast; b is then the outer
// block (nbatch = outer blocks x inner). Contiguous sequences (inner == 1)
// take chunks fastest.
struct SolveLane {
  int64_t b, ch, i, rs;
};
__device__ __forceinline__ SolveLane solve_lane(const SolveParams& sp, int64_t tid) {
  SolveLane l;
  if (sp.inner > 1) {
    const int64_t r = tid / sp.inner;
    l.i = tid - r * sp.inner;
    l.b = r / sp.nchunk;
    l.ch = r - l.b * sp.nchunk;
    l.rs = sp.inner;
  } else {
    l.b = tid / sp.nchunk;
    l.ch = tid - l.b * sp.nchunk;
    l.i = 0;
    l.rs = 1;
  }
  return l;
}

// HvdH banded solve (FFTJ _hvdh_subst! / _hvdh_back!, src/hvdh.jl:604-686):
// thread (b, c) runs forward substitution over its chunk's R rows (rows q0
// .. q0+R-1 of the length-t transform, cyclic), keeping z in a strided
// scratch, then back substitution, writing the core rows' unknowns to their
// permuted outputs, scaled by scale * n / t.
// HvdH banded solve with its factors rebuilt per call (FFTJ factors = :fly,
// src/hvdh.jl:500-602): thread (b, c) walks its chunk's R rows; column j's
// state e_j = 2 t l' - 2 n q_j + n (an unknown sits at row q_j when
// e_j < 2n, offset beta' = (e_j - n)/2n; the next column's state is e + 2
// Delta on an unknown, e - 2n off one) gives row i's band entries
// exp(-a (k + beta'_{i+k})^2), |k| <= B, columns outside [0, R) dropped as
// in the tabulated factors; rows are eliminated without pivoting as they are
// built, their U rows and output indices kept in per-thread scratch for the
// back pass. Same mathematics as the tabulated solve (solve_at), FP64 exp
// per column instead of a table read per row: on GB300 (slow FP64, fast
// HBM) the tables are faster, so they are the default up to a size cap.
template <typename T, int B, bool CG>
__device__ __forceinline__ void solve_fly_at(const SolveParams& sp, const Cx<T>* __restrict__ g,
                                             Cx<T>* __restrict__ y, const int64_t tid) {
  const int64_t nt = sp.nbatch * sp.nchunk;
  if (tid >= nt) return;
  const SolveLane ln = solve_lane(sp, tid);
  const int64_t b = ln.b, ch = ln.ch, rs = ln.rs;
  const int R = (int)sp.R, H = (int)sp.H, L = (int)sp.L;
  const int t = (int)sp.t;
  const int64_t n = sp.n, d2 = 2 * sp.delta, n2 = 2 * n;
  const double a = sp.a, inv2n = 1.0 / (double)n2;
  constexpr int W = 2 * B + 1;
  // column window: columns i - B .. i + B of row i (relative to the chunk)
  int64_t e = sp.se[ch];
  double beta[W];
  bool hit[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    hit[w] = e < n2;
    beta[w] = (double)(e - n) * inv2n;
    e = hit[w] ? e + d2 : e - n2;
  }
  int64_t on = sp.so[ch];
  Cx<T>* zwp = reinterpret_cast<Cx<T>*>(sp.zw) + tid;
  T* uwp = reinterpret_cast<T*>(sp.uw) + tid;
  int32_t* owp = sp.ow + tid;
  const Cx<T>* gb = g + b * sp.g_bstride + ln.i;
  int q = (int)((((int64_t)ch * L - H) % t + t) % t);
  T up[B][B + 1];  // U rows i-1 .. i-B: 1/U_jj, U_{j,j+1..j+B}
#pragma unroll
  for (int k = 0; k < B; ++k) {
    up[k][0] = (T)1;
#pragma unroll
    for (int j = 1; j <= B; ++j) up[k][j] = (T)0;
  }
  Cx<T> zp[B];
#pragma unroll
  for (int k = 0; k < B; ++k) zp[k] = mk<T>(0, 0);
  for (int i = 0; i < R; ++i) {
    // row i's band: r[k + B] = entry at column i + k
    T r[W];
    const bool hi = hit[B];
#pragma unroll
    for (int k = -B; k <= B; ++k) {
      const int j = i + k;
      const double dd = (double)k + beta[k + B];
      r[k + B] = (hi && hit[k + B] && j >= 0 && j < R) ? (T)exp(-a * dd * dd) : (T)0;
    }
    if (!hi) r[B] = (T)1;  // identity row
    // eliminate columns i-B .. i-1 against the previous U rows
    Cx<T> z = mk<T>(0, 0);
    if (hi) z = ldd<CG>(gb + (int64_t)q * rs);
#pragma unroll
    for (int k = B; k >= 1; --k) {
      const T f = r[B - k] * up[k - 1][0];
#pragma unroll
      for (int j = 1; j <= B; ++j) r[B - k + j] = fma(-f, up[k - 1][j], r[B - k + j]);
      z.x = fma(-f, zp[k - 1].x, z.x);
      z.y = fma(-f, zp[k - 1].y, z.y);
    }
#pragma unroll
    for (int k = B - 1; k > 0; --k) {
      zp[k] = zp[k - 1];
#pragma unroll
      for (int j = 0; j <= B; ++j) up[k][j] = up[k - 1][j];
    }
    zp[0] = z;
    up[0][0] = (T)1 / r[B];
#pragma unroll
    for (int j = 1; j <= B; ++j) up[0][j] = r[B + j];
    zwp[(int64_t)i * nt] = z;
#pragma unroll
    for (int j = 0; j <= B; ++j) uwp[((int64_t)i * (B + 1) + j) * nt] = up[0][j];
    owp[(int64_t)i * nt] = hi ? (int32_t)on : -1;
    if (hi) { on += sp.delta; if (on >= n) on -= n; }
    // slide the column window by one
#pragma unroll
    for (int w = 0; w < W - 1; ++w) { hit[w] = hit[w + 1]; beta[w] = beta[w + 1]; }
    hit[W - 1] = e < n2;
    beta[W - 1] = (double)(e - n) * inv2n;
    e = hit[W - 1] ? e + d2 : e - n2;
    if (++q >= t) q -= t;
  }
  // back substitution from row R-1 down to H
  Cx<T> xp[B];
#pragma unroll
  for (int k = 0; k < B; ++k) xp[k] = mk<T>(0, 0);
  const T sc = (T)sp.sc;
  Cx<T>* yb = y + b * sp.y_bstride + ln.i;
  const Cx<T>* twb = sp.tw ? reinterpret_cast<const Cx<T>*>(sp.tw) : nullptr;
  const int64_t twr = sp.tw ? (b % sp.tw_s) : 0;
  for (int i = R - 1; i >= H; --i) {
    Cx<T> x = zwp[(int64_t)i * nt];
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const T u = uwp[((int64_t)i * (B + 1) + 1 + j) * nt];
      x.x = fma(-u, xp[j].x, x.x);
      x.y = fma(-u, xp[j].y, x.y);
    }
    const T iu = uwp[(int64_t)i * (B + 1) * nt];
    x.x *= iu;
    x.y *= iu;
#pragma unroll
    for (int k = B - 1; k > 0; --k) xp[k] = xp[k - 1];
    xp[0] = x;
    const int32_t o = owp[(int64_t)i * nt];
    if (i < H + L && o >= 0) {
      Cx<T> v = mk<T>(x.x * sc, x.y * sc);
      if (twb) v = cmul(v, __ldg(twb + twr * o));
      yb[(int64_t)o * rs] = v;
    }
  }
}

template <typename T, int B, bool CG, int K = 8>
__device__ __forceinline__ void solve_at(const SolveParams& sp, const Cx<T>* __restrict__ g,
                                         Cx<T>* __restrict__ y, const int64_t tid) {
  // Rows go in blocks of K: a block's operands (input rows, LU factors,
  // output indices) are loaded together, then its K dependent recurrence
  // steps run from registers. Row pointers advance by increments (the
  // kernel is a latency chain: every instruction of a row counts). The
  // persistent group kernel (128 registers a thread) takes K = 4.
  const int64_t nt = sp.nbatch * sp.nchunk;
  if (tid >= nt) return;
  const SolveLane ln = solve_lane(sp, tid);
  const int64_t b = ln.b, ch = ln.ch, rs = ln.rs;
  const int R = (int)sp.R, H = (int)sp.H, L = (int)sp.L;
  const int t = (int)sp.t;
  // factor tables are row-major across chunks: row i of chunk ch at
  // i * nchunk + ch (adjacent lanes read adjacent entries)
  const int64_t nc = sp.nchunk;
  const T* lfp = reinterpret_cast<const T*>(sp.lf) + ch * B;
  const T* ufp = reinterpret_cast<const T*>(sp.uf) + ch * (B + 1);
  const int32_t* oip = sp.oi + ch;
  const int64_t lstep = nc * B, ustep = nc * (B + 1);
  Cx<T>* zwp = reinterpret_cast<Cx<T>*>(sp.zw) + tid;
  const Cx<T>* gb = g + b * sp.g_bstride + ln.i;
  int q = (int)((((int64_t)ch * L - H) % t + t) % t);
  Cx<T> zp[B];
#pragma unroll
  for (int k = 0; k < B; ++k) zp[k] = mk<T>(0, 0);  // zp[k] = z_{i-1-k}
  for (int i0 = 0; i0 < R; i0 += K) {
    Cx<T> gv[K];
    T f[K][B];
#pragma unroll
    for (int u = 0; u < K; ++u) {
      gv[u] = mk<T>(0, 0);
      if (i0 + u < R) {
        int qq = q + u;
        if (qq >= t) qq -= t;
        const Cx<T> v = ldd<CG>(gb + (int64_t)qq * rs);  // in range for every row: load, then mask
        if (__ldg(oip + u * nc) >= 0) gv[u] = v;
#pragma unroll
        for (int k = 0; k < B; ++k) f[u][k] = __ldg(lfp + u * lstep + k);
      }
    }
#pragma unroll
    for (int u = 0; u < K; ++u) {
      if (i0 + u < R) {
        Cx<T> z = gv[u];
#pragma unroll
        for (int k = 0; k < B; ++k) {
          z.x = fma(-f[u][k], zp[k].x, z.x);
          z.y = fma(-f[u][k], zp[k].y, z.y);
        }
#pragma unroll
        for (int k = B - 1; k > 0; --k) zp[k] = zp[k - 1];
        zp[0] = z;
        zwp[u * nt] = z;
      }
    }
    q += K;
    if (q >= t) q -= t;
    lfp += K * lstep;
    oip += K * nc;
    zwp += K * nt;
  }
  Cx<T> xp[B];
#pragma unroll
  for (int k = 0; k < B; ++k) xp[k] = mk<T>(0, 0);  // xp[k] = x_{i+1+k}
  const T sc = (T)sp.sc;
  Cx<T>* yb = y + b * sp.y_bstride + ln.i;
  const Cx<T>* twb = sp.tw ? reinterpret_cast<const Cx<T>*>(sp.tw) + 0 : nullptr;
  const int64_t twr = sp.tw ? (b % sp.tw_s) : 0;
  // back substitution from row R-1 down to H
  const Cx<T>* zr = reinterpret_cast<const Cx<T>*>(sp.zw) + tid + (int64_t)(R - 1) * nt;
  const T* urp = reinterpret_cast<const T*>(sp.uf) + ch * (B + 1) + (int64_t)(R - 1) * ustep;
  const int32_t* orp = sp.oi + ch + (int64_t)(R - 1) * nc;
  for (int i0 = R - 1; i0 >= H; i0 -= K) {
    Cx<T> zv[K];
    T uu[K][B + 1];
    int32_t ov[K];
#pragma unroll
    for (int u = 0; u < K; ++u) {
      if (i0 - u >= H) {
        zv[u] = zr[-(int64_t)u * nt];
#pragma unroll
        for (int j = 0; j <= B; ++j) uu[u][j] = __ldg(urp - u * ustep + j);
        ov[u] = __ldg(orp - u * nc);
      }
    }
#pragma unroll
    for (int u = 0; u < K; ++u) {
      const int i = i0 - u;
      if (i >= H) {
        Cx<T> x = zv[u];
#pragma unroll
        for (int j = 0; j < B; ++j) {
          x.x = fma(-uu[u][1 + j], xp[j].x, x.x);
          x.y = fma(-uu[u][1 + j], xp[j].y, x.y);
        }
        x.x *= uu[u][0];
        x.y *= uu[u][0];
#pragma unroll
        for (int k = B - 1; k > 0; --k) xp[k] = xp[k - 1];
        xp[0] = x;
        const int32_t o = ov[u];
        if (i < H + L && o >= 0) {
          Cx<T> v = mk<T>(x.x * sc, x.y * sc);
          if (twb) v = cmul(v, __ldg(twb + twr * o));
          yb[(int64_t)o * rs] = v;
        }
      }
    }
    zr -= K * nt;
    urp -= K * ustep;
    orp -= K * nc;
  }
}

// rfft even post-pass (FFTJ src/real.jl:85-135): X[k] = xe + w (-i xo).
// X[k] and X[h-k] both come from Z[k] and Z[h-k], so one thread makes the
// pair (k = 0 .. h/2, k = 0 also writing X[h]) and each Z entry is read once.
template <typename T>
__device__ __forceinline__ Cx<T> real_post_one(Cx<T> a, Cx<T> bb, Cx<T> w) {
  bb.y = -bb.y;  // conj Z[h - k]
  const T half = (T)0.5;
  const T xer = (a.x + bb.x) * half, xei = (a.y + bb.y) * half;
  const T xor_ = (a.x - bb.x) * half, xoi = (a.y - bb.y) * half;
  return mk<T>(xer + fma(w.x, xoi, w.y * xor_), xei + fma(w.y, xoi, -(w.x * xor_)));
}

template <typename T, bool CG>
__device__ __forceinline__ void real_post_at(const RealPostParams& rp, const Cx<T>* __restrict__ z,
                                             Cx<T>* __restrict__ y, const int64_t idx) {
  const int64_t h = rp.h, nk = h / 2 + 1;
  if (idx >= nk * rp.nbatch) return;
  const int64_t b = idx / nk, k = idx - b * nk;
  const Cx<T>* Z = z + b * rp.z_bstride;
  Cx<T>* Y = y + b * rp.y_bstride;
  const Cx<T>* tw = reinterpret_cast<const Cx<T>*>(rp.tw);
  if (k == 0) {
    const Cx<T> z0 = ldd<CG>(Z);
    Y[0] = mk<T>(z0.x + z0.y, 0);
    Y[h] = mk<T>(z0.x - z0.y, 0);
    return;
  }
  const Cx<T> a = ldd<CG>(Z + k);
  const Cx<T> m = ldd<CG>(Z + (h - k));
  // w^k (k <= h/2) from the table or its two-level split; the mirror's
  // twiddle is w^(h-k) = -conj(w^k) (n = 2h), exact in any precision
  Cx<T> w;
  if (rp.sh) {
    const Cx<T> hi = __ldg(tw + (k >> rp.sh));
    const Cx<T> lo = __ldg(reinterpret_cast<const Cx<T>*>(rp.tw2) + (k & ((1ll << rp.sh) - 1)));
    w = cmul(hi, lo);
  } else {
    w = __ldg(tw + k);
  }
  Y[k] = real_post_one<T>(a, m, w);
  if (h - k != k) Y[h - k] = real_post_one<T>(m, a, mk<T>(-w.x, w.y));
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
  } else if (cp.mode == 6) {
    // CompositePlan's twiddle and transpose (src/composite.jl:93-96, the
    // twiddles fused into the next pass as FFTJ fuses them into its
    // deconvolution): output (j1, k2) at k2 + s j1 = input (k2, j1) at
    // j1 + p k2, times w_n^(j1 k2) (j1 k2 < n)
    const int64_t sd = cp.nc, pl = cp.n / sd;
    const int64_t j1 = j / sd, k2 = j - j1 * sd;
    const Cx<T> v = ldd<CG>(reinterpret_cast<const Cx<T>*>(in) + b * cp.in_bstride + j1 + pl * k2);
    const Cx<T> w = __ldg(reinterpret_cast<const Cx<T>*>(cp.tab) + j1 * k2);
    reinterpret_cast<Cx<T>*>(out)[b * cp.out_bstride + j] = cmul(v, w);
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
