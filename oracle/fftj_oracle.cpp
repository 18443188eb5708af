// TEST INFRASTRUCTURE ONLY — the oracle. Never part of the product path.
//
// CPU restatement of FFTJ.jl's transform path (oscardssmith/FFTJ.jl, pure
// Julia; Julia is absent here so the reference cannot be run). Every function
// cites the reference file:line it follows. The scalar branches of FFTJ's
// SIMD stage loops give the canonical index maps restated here; the loops over
// the stride lane q are left to the compiler's auto-vectoriser (NEON on the
// Grace host), standing in for FFTJ's explicit SIMD.Vec code.
//
// Parity status: parity unpinned -- the reference's tests hold no stored
// vectors (they draw random inputs and call FFTW at run time) and the
// reference cannot be run here, so this restatement is checked against an
// FP64 direct DFT (double-double accumulation, exact angle reduction) and
// numpy's pocketfft at the reference test sizes and tolerance classes, not
// against reference outputs; see tests/test_oracle.py.
#include "fftj_oracle.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace orc {

using i64 = int64_t;

// ---------------------------------------------------------------------------
// Host SIMD width (src/kernels.jl:11-22): only used for routing and towers.
static int g_vector_bits = 128;
template <typename T>
static inline int pick_width() { return g_vector_bits / (8 * (int)sizeof(T)); }

// ---------------------------------------------------------------------------
// sin(pi x), cos(pi x) with exact reduction to [0, 1/4] (stands in for
// Julia's Base.sincospi used for every twiddle, src/plan.jl:76-77).
static void sincospi(double x, double* s, double* c) {
  double sg = 1.0;
  if (x < 0) { x = -x; sg = -1.0; }
  double r = std::fmod(x, 2.0);
  double ss = 1.0, cs = 1.0;
  if (r >= 1.0) { r -= 1.0; ss = -ss; cs = -cs; }
  bool swap = false;
  if (r > 0.5) { r = 1.0 - r; cs = -cs; }
  if (r > 0.25) { r = 0.5 - r; swap = true; }
  double a = M_PI * r;
  double sv = std::sin(a), cv = std::cos(a);
  if (swap) std::swap(sv, cv);
  *s = sg * ss * sv;
  *c = cs * cv;
}
static inline double cospi_(double x) { double s, c; sincospi(x, &s, &c); return c; }
static inline double sinpi_(double x) { double s, c; sincospi(x, &s, &c); return s; }

// ---------------------------------------------------------------------------
// Deterministic fork-join (src/threads.jl:15-41): split [0, len) into at most
// nt chunks whose starts sit on `align`; the last chunk absorbs the tail.
class Pool {
 public:
  static Pool& get() { static Pool p; return p; }
  int size() const { return (int)workers_.size() + 1; }
  // run f(ci) for ci in [0, nchunks) on the workers and the caller
  void run(int nchunks, const std::function<void(int)>& f) {
    if (nchunks <= 1) { if (nchunks == 1) f(0); return; }
    std::unique_lock<std::mutex> lk(mu_);
    job_ = &f;
    njob_ = nchunks;
    next_.store(1);
    done_ = 0;
    gen_++;
    cv_.notify_all();
    lk.unlock();
    f(0);
    for (;;) {
      int c = next_.fetch_add(1);
      if (c >= nchunks) break;
      f(c);
      std::lock_guard<std::mutex> g(mu_);
      done_++;
    }
    lk.lock();
    done_cv_.wait(lk, [&] { return done_ >= nchunks - 1; });
    job_ = nullptr;
  }
  ~Pool() {
    { std::lock_guard<std::mutex> g(mu_); stop_ = true; gen_++; }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }

 private:
  Pool() {
    unsigned hc = std::thread::hardware_concurrency();
    int nw = (int)(hc > 1 ? hc - 1 : 0);
    for (int i = 0; i < nw; ++i) workers_.emplace_back([this] { loop(); });
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      const std::function<void(int)>* job;
      int nj;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
        job = job_;
        nj = njob_;
      }
      if (!job) continue;
      for (;;) {
        int c = next_.fetch_add(1);
        if (c >= nj) break;
        (*job)(c);
        std::lock_guard<std::mutex> g(mu_);
        done_++;
        if (done_ >= nj - 1) done_cv_.notify_all();
      }
    }
  }
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* job_ = nullptr;
  int njob_ = 0;
  std::atomic<int> next_{0};
  int done_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// tforeach_chunks (src/threads.jl:15-38), 0-based half-open ranges.
static void tforeach_chunks(i64 len, int nt, i64 align,
                            const std::function<void(int, i64, i64)>& f) {
  if (len <= 0) return;
  i64 units = len / align;
  i64 nchunks = std::min<i64>(nt, units);
  if (nchunks <= 1) { f(0, 0, len); return; }
  i64 per = units / nchunks, rem = units % nchunks;
  std::vector<i64> lo(nchunks), hi(nchunks);
  i64 l = 0;
  for (i64 c = 0; c < nchunks; ++c) {
    i64 u = per + (c < rem ? 1 : 0);
    i64 h = (c == nchunks - 1) ? len : l + u * align;
    lo[c] = l; hi[c] = h; l = h;
  }
  Pool::get().run((int)nchunks, [&](int c) { f(c, lo[c], hi[c]); });
}
static void tforeach(i64 len, int nt, i64 align, const std::function<void(i64, i64)>& f) {
  tforeach_chunks(len, nt, align, [&](int, i64 lo, i64 hi) { f(lo, hi); });
}
static const i64 MIN_CHUNK = 1 << 15;  // src/threads.jl:7
static int plan_tasks(i64 work, int nthreads) {  // src/plan.jl:62
  return (int)std::min<i64>(std::max(nthreads, 1), std::max<i64>(work / MIN_CHUNK, 1));
}

// ---------------------------------------------------------------------------
// Factorization (src/plan.jl:16-45).
static const int ODD_RADICES[5] = {13, 11, 7, 5, 3};
struct Fac { int a; std::vector<std::pair<int, int>> ps; bool ok; };
static Fac factor_radices(i64 n) {
  Fac f; f.ok = false; f.a = 0;
  if (n < 1) return f;
  int a = __builtin_ctzll((unsigned long long)n);
  i64 r = n >> a;
  for (int p : ODD_RADICES) {
    int c = 0;
    while (r % p == 0) { r /= p; c++; }
    if (c > 0) f.ps.push_back({p, c});
  }
  f.a = a;
  f.ok = (r == 1);
  return f;
}
static bool factor_smooth(i64 n) {
  if (n < 1) return false;
  i64 r = n >> __builtin_ctzll((unsigned long long)n);
  for (int p : {3, 5, 7}) while (r % p == 0) r /= p;
  return r == 1;
}

template <typename T>
struct Stage {
  int radix;
  std::vector<T> twr, twi;  // (radix-1) twiddles per butterfly, [(radix-1)*p + j-1]
};

// make_stage (src/plan.jl:66-95), non-small layout (same values).
template <typename T>
static Stage<T> make_stage(int radix, i64 n, int D) {
  i64 m = n / radix;
  Stage<T> st;
  st.radix = radix;
  st.twr.resize((size_t)(radix - 1) * m);
  st.twi.resize((size_t)(radix - 1) * m);
  for (i64 p = 0; p < m; ++p)
    for (int j = 1; j < radix; ++j) {
      double th = (double)(2 * D * p * j) / (double)n;
      double s, c;
      sincospi(th, &s, &c);
      st.twr[(size_t)(radix - 1) * p + j - 1] = (T)c;
      st.twi[(size_t)(radix - 1) * p + j - 1] = (T)s;
    }
  return st;
}

// _tower (src/plan.jl:105-117)
template <typename T>
static void tower(int a, bool allow_small, int* f, std::vector<int>* rad) {
  rad->clear();
  if (a == 0) { *f = 1; return; }
  if (a <= 3) { *f = 1 << a; return; }
  int W = pick_width<T>();
  int k = 0;
  while (allow_small && (1 << (2 * k)) < W && 2 * (k + 1) <= a - 2) k++;
  int b = a - 2 * k;
  const int n4tab[3] = {0, 2, 1};
  int n4 = n4tab[b % 3];
  std::vector<int> r;
  for (int i = 0; i < k + n4; ++i) r.push_back(4);
  for (int i = 0; i < (b - 2 * n4) / 3; ++i) r.push_back(8);
  *f = r.back();
  r.pop_back();
  *rad = r;
}

// build_stages (src/plan.jl:125-151): tower, odd stages smallest first, final f.
template <typename T>
static std::vector<Stage<T>> build_stages(i64 n, int D, bool allow_small, int* fout = nullptr) {
  Fac fac = factor_radices(n);
  if (!fac.ok) throw std::runtime_error("build_stages requires 13-smooth n");
  int f;
  std::vector<int> tw;
  tower<T>(fac.a, allow_small, &f, &tw);
  std::vector<Stage<T>> stages;
  i64 ncur = n;
  for (int r : tw) { stages.push_back(make_stage<T>(r, ncur, D)); ncur /= r; }
  for (auto it = fac.ps.rbegin(); it != fac.ps.rend(); ++it)
    for (int c = 0; c < it->second; ++c) {
      stages.push_back(make_stage<T>(it->first, ncur, D));
      ncur /= it->first;
    }
  if (f > 1) stages.push_back(make_stage<T>(f, ncur, D));
  if (fout) *fout = f;
  return stages;
}

// ---------------------------------------------------------------------------
// Butterflies (src/kernels.jl:24-239), scalar.
template <typename T>
static inline void cmul(T wr, T wi, T xr, T xi, T* yr, T* yi) {
  *yr = std::fma(wr, xr, -(wi * xi));
  *yi = std::fma(wr, xi, wi * xr);
}

template <typename T>
static inline void bf4_core(T ar, T ai, T br, T bi, T cr, T ci, T dr, T di, int D, T* y) {
  T apcr = ar + cr, apci = ai + ci, amcr = ar - cr, amci = ai - ci;
  T bpdr = br + dr, bpdi = bi + di, bmdr = br - dr, bmdi = bi - di;
  y[0] = apcr + bpdr; y[1] = apci + bpdi;
  if (D == -1) {
    y[2] = amcr + bmdi; y[3] = amci - bmdr;
    y[6] = amcr - bmdi; y[7] = amci + bmdr;
  } else {
    y[2] = amcr - bmdi; y[3] = amci + bmdr;
    y[6] = amcr + bmdi; y[7] = amci - bmdr;
  }
  y[4] = apcr - bpdr; y[5] = apci - bpdi;
}

template <typename T>
static inline void bf8_core(const T* xr, const T* xi, T c, int D, T* y) {
  T e[8], o[8];
  bf4_core(xr[0], xi[0], xr[2], xi[2], xr[4], xi[4], xr[6], xi[6], D, e);
  bf4_core(xr[1], xi[1], xr[3], xi[3], xr[5], xi[5], xr[7], xi[7], D, o);
  T t1r, t1i, t2r, t2i, t3r, t3i;
  if (D == -1) {
    t1r = c * (o[2] + o[3]); t1i = c * (o[3] - o[2]);
    t2r = o[5]; t2i = -o[4];
    t3r = c * (o[7] - o[6]); t3i = -c * (o[6] + o[7]);
  } else {
    t1r = c * (o[2] - o[3]); t1i = c * (o[3] + o[2]);
    t2r = -o[5]; t2i = o[4];
    t3r = -c * (o[6] + o[7]); t3i = c * (o[6] - o[7]);
  }
  y[0] = e[0] + o[0]; y[1] = e[1] + o[1];
  y[2] = e[2] + t1r; y[3] = e[3] + t1i;
  y[4] = e[4] + t2r; y[5] = e[5] + t2i;
  y[6] = e[6] + t3r; y[7] = e[7] + t3i;
  y[8] = e[0] - o[0]; y[9] = e[1] - o[1];
  y[10] = e[2] - t1r; y[11] = e[3] - t1i;
  y[12] = e[4] - t2r; y[13] = e[5] - t2i;
  y[14] = e[6] - t3r; y[15] = e[7] - t3i;
}

// bfp_consts / bfp (src/kernels.jl:158-228): odd-prime DFT by conjugate pairs.
template <typename T>
struct BfpConsts {
  int P, h;
  std::vector<T> cc, ss;  // [(k-1)*h + (j-1)]
  BfpConsts(int P_, int D) : P(P_), h((P_ - 1) / 2) {
    cc.resize(h * h); ss.resize(h * h);
    for (int k = 1; k <= h; ++k)
      for (int j = 1; j <= h; ++j) {
        double th = (double)(2 * (j * k)) / (double)P;
        cc[(k - 1) * h + j - 1] = (T)cospi_(th);
        ss[(k - 1) * h + j - 1] = (T)(D * sinpi_(th));
      }
  }
};

template <typename T>
static inline void bfp(int P, const T* xr, const T* xi, const BfpConsts<T>& K, T* yr, T* yi) {
  int h = (P - 1) / 2;
  T tr[6], ti[6], dr[6], di[6];
  for (int j = 1; j <= h; ++j) {
    tr[j - 1] = xr[j] + xr[P - j]; ti[j - 1] = xi[j] + xi[P - j];
    dr[j - 1] = xr[j] - xr[P - j]; di[j - 1] = xi[j] - xi[P - j];
  }
  T sr = tr[0], si = ti[0];
  for (int j = 2; j <= h; ++j) { sr = sr + tr[j - 1]; si = si + ti[j - 1]; }
  yr[0] = xr[0] + sr; yi[0] = xi[0] + si;
  for (int k = 1; k <= h; ++k) {
    T er = xr[0], ei = xi[0];
    for (int j = h; j >= 1; --j) {
      T c = K.cc[(k - 1) * h + j - 1];
      er = std::fma(c, tr[j - 1], er);
      ei = std::fma(c, ti[j - 1], ei);
    }
    T s = K.ss[(k - 1) * h + h - 1];
    T vr = s * dr[h - 1], vi = s * di[h - 1];
    for (int j = h - 1; j >= 1; --j) {
      T sj = K.ss[(k - 1) * h + j - 1];
      vr = std::fma(sj, dr[j - 1], vr);
      vi = std::fma(sj, di[j - 1], vi);
    }
    yr[k] = er - vi; yi[k] = ei + vr;          // X_k = u + i v
    yr[P - k] = er + vi; yi[P - k] = ei - vr;  // X_{P-k} = u - i v
  }
}

// ---------------------------------------------------------------------------
// Stage loops (src/stockham.jl:26-428), scalar index maps over p in
// [plo, phi) and q in [qlo, qhi): read x[s*p + j*m*s + q], write
// y[r*s*p + j*s + q] twiddled by w_j (output 0 untwiddled).
template <typename T>
static void run_stage_pq(T* yre, T* yim, const T* xre, const T* xim, i64 n, i64 s,
                         const Stage<T>& st, int D, i64 plo, i64 phi, i64 qlo, i64 qhi) {
  const int r = st.radix;
  const i64 m = n / r, ms = m * s;
  const T* twr = st.twr.data();
  const T* twi = st.twi.data();
  if (r == 4) {
    for (i64 p = plo; p < phi; ++p) {
      T w1r = twr[3 * p], w1i = twi[3 * p], w2r = twr[3 * p + 1], w2i = twi[3 * p + 1];
      T w3r = twr[3 * p + 2], w3i = twi[3 * p + 2];
      i64 xb = s * p, yb = 4 * s * p;
      for (i64 q = qlo; q < qhi; ++q) {
        T y[8];
        bf4_core(xre[xb + q], xim[xb + q], xre[xb + ms + q], xim[xb + ms + q],
                 xre[xb + 2 * ms + q], xim[xb + 2 * ms + q], xre[xb + 3 * ms + q],
                 xim[xb + 3 * ms + q], D, y);
        yre[yb + q] = y[0]; yim[yb + q] = y[1];
        cmul(w1r, w1i, y[2], y[3], &yre[yb + s + q], &yim[yb + s + q]);
        cmul(w2r, w2i, y[4], y[5], &yre[yb + 2 * s + q], &yim[yb + 2 * s + q]);
        cmul(w3r, w3i, y[6], y[7], &yre[yb + 3 * s + q], &yim[yb + 3 * s + q]);
      }
    }
  } else if (r == 8) {
    const T c = (T)std::sqrt(0.5);
    for (i64 p = plo; p < phi; ++p) {
      i64 xb = s * p, yb = 8 * s * p;
      for (i64 q = qlo; q < qhi; ++q) {
        T xr[8], xi[8], y[16];
        for (int k = 0; k < 8; ++k) { xr[k] = xre[xb + k * ms + q]; xi[k] = xim[xb + k * ms + q]; }
        bf8_core(xr, xi, c, D, y);
        yre[yb + q] = y[0]; yim[yb + q] = y[1];
        for (int j = 1; j < 8; ++j)
          cmul(twr[7 * p + j - 1], twi[7 * p + j - 1], y[2 * j], y[2 * j + 1],
               &yre[yb + j * s + q], &yim[yb + j * s + q]);
      }
    }
  } else if (r == 2) {
    for (i64 p = plo; p < phi; ++p) {
      T wr = twr[p], wi = twi[p];
      i64 xb = s * p, yb = 2 * s * p;
      for (i64 q = qlo; q < qhi; ++q) {
        T ar = xre[xb + q], ai = xim[xb + q], br = xre[xb + ms + q], bi = xim[xb + ms + q];
        yre[yb + q] = ar + br; yim[yb + q] = ai + bi;
        cmul(wr, wi, ar - br, ai - bi, &yre[yb + s + q], &yim[yb + s + q]);
      }
    }
  } else {
    BfpConsts<T> K(r, D);
    for (i64 p = plo; p < phi; ++p) {
      i64 xb = s * p, yb = r * s * p;
      for (i64 q = qlo; q < qhi; ++q) {
        T xr[13], xi[13], yr[13], yi[13];
        for (int j = 0; j < r; ++j) { xr[j] = xre[xb + j * ms + q]; xi[j] = xim[xb + j * ms + q]; }
        bfp(r, xr, xi, K, yr, yi);
        yre[yb + q] = yr[0]; yim[yb + q] = yi[0];
        for (int j = 1; j < r; ++j)
          cmul(twr[(r - 1) * p + j - 1], twi[(r - 1) * p + j - 1], yr[j], yi[j],
               &yre[yb + j * s + q], &yim[yb + j * s + q]);
      }
    }
  }
}

// run_stage! / run_stage_par! (src/plan.jl:215-284): split butterflies p when
// plentiful, else W-aligned lanes q.
template <typename T>
static void run_stage(T* yre, T* yim, const T* xre, const T* xim, i64 n, i64 s,
                      const Stage<T>& st, int D, int nt) {
  i64 m = n / st.radix;
  if (nt <= 1) { run_stage_pq(yre, yim, xre, xim, n, s, st, D, 0, m, 0, s); return; }
  int W = pick_width<T>();
  if (m >= nt || s < W) {
    tforeach(m, nt, 1, [&](i64 lo, i64 hi) { run_stage_pq(yre, yim, xre, xim, n, s, st, D, lo, hi, 0, s); });
  } else {
    tforeach(s, nt, W, [&](i64 lo, i64 hi) { run_stage_pq(yre, yim, xre, xim, n, s, st, D, 0, m, lo, hi); });
  }
}

// run_chain! (src/plan.jl:311-321): ping-pong, effective stride s*B.
// Returns true when the result sits in (ore, oim).
template <typename T>
static bool run_chain(T* cre, T* cim, T* ore, T* oim, const std::vector<Stage<T>>& stages,
                      size_t from, size_t to, i64 ncur, i64 s, i64 B, int D, int nt) {
  bool swapped = false;
  for (size_t k = from; k < to; ++k) {
    const Stage<T>& st = stages[k];
    run_stage(ore, oim, cre, cim, ncur, s * B, st, D, nt);
    std::swap(cre, ore); std::swap(cim, oim);
    swapped = !swapped;
    s *= st.radix;
    ncur /= st.radix;
  }
  return swapped;
}

// ---------------------------------------------------------------------------
// Plans.
struct PlanBase {
  virtual ~PlanBase() {}
  int route = ORC_FFTPLAN;
  i64 n = 0;
  virtual void exec(const void* x, void* y) = 0;
  virtual void info(std::vector<i64>& v) { v.push_back(route); v.push_back(n); }
};

template <typename T>
static T default_scale(i64 n, int D) { return D == -1 ? (T)1 : (T)1 / (T)n; }  // src/plan.jl:97

// FFTPlan (src/plan.jl:48-58, 169-177, 359-396).
template <typename T>
struct FFTPlan : PlanBase {
  int D;
  T scale;
  int nt;
  std::vector<Stage<T>> stages;
  std::vector<T> are, aim, bre, bim;
  FFTPlan(i64 n_, int D_, T scale_, int nthreads) : D(D_), scale(scale_) {
    n = n_;
    route = ORC_FFTPLAN;
    stages = build_stages<T>(n, D, true);
    are.resize(n); aim.resize(n); bre.resize(n); bim.resize(n);
    nt = plan_tasks(n, nthreads);
  }
  // planes in -> planes out (result pointer returned)
  void exec(const void* xv, void* yv) override {
    const T* x = (const T*)xv;
    T* y = (T*)yv;
    // deinterleave_all! (src/stockham.jl:448-469)
    tforeach(n, nt, pick_width<T>(), [&](i64 lo, i64 hi) {
      for (i64 c = lo; c < hi; ++c) { are[c] = x[2 * c]; aim[c] = x[2 * c + 1]; }
    });
    bool sw = run_chain(are.data(), aim.data(), bre.data(), bim.data(), stages, 0, stages.size(),
                        n, 1, 1, D, nt);
    const T* rr = sw ? bre.data() : are.data();
    const T* ri = sw ? bim.data() : aim.data();
    // interleave_all! with scale (src/stockham.jl:486-506)
    T sc = scale;
    tforeach(n, nt, pick_width<T>(), [&](i64 lo, i64 hi) {
      for (i64 c = lo; c < hi; ++c) { y[2 * c] = rr[c] * sc; y[2 * c + 1] = ri[c] * sc; }
    });
  }
  void info(std::vector<i64>& v) override {
    v.push_back(route); v.push_back(n);
    for (auto& s : stages) v.push_back(s.radix);
  }
};

// ---- four-step (src/fourstep.jl) ------------------------------------------
static const i64 FS_INNER_MAX = 1 << 19;  // src/fourstep.jl:40
static const i64 FS_TASK_MIN = 1 << 13;   // src/fourstep.jl:251

// _fs_pick (src/fourstep.jl:184-199)
static i64 fs_pick(i64 n, i64 S, i64 t) {
  i64 best = 0, besttile = 0;
  auto dist = [&](i64 d) { return std::fabs(std::log((double)d / (double)t)); };
  auto better = [&](i64 d, i64 b) { return b == 0 || dist(d) < dist(b) || (dist(d) == dist(b) && d < b); };
  i64 rq = (i64)std::sqrt((double)n);
  while (rq * rq > n) rq--;
  while ((rq + 1) * (rq + 1) <= n) rq++;
  for (i64 q = 1; q <= rq; ++q) {
    if (n % q) continue;
    i64 ds[2] = {q, n / q};
    for (i64 d : ds) {
      if (!(d >= S && n / d >= S)) continue;
      if (!factor_radices(d).ok || !factor_radices(n / d).ok) continue;
      if (better(d, best)) best = d;
      if (d % S == 0 && (n / d) % S == 0 && dist(d) <= std::log(2.0) && better(d, besttile)) besttile = d;
    }
  }
  return besttile != 0 ? besttile : best;
}
static i64 isqrt_(i64 n) {
  i64 r = (i64)std::sqrt((double)n);
  while (r * r > n) r--;
  while ((r + 1) * (r + 1) <= n) r++;
  return r;
}

// _fourstep_split (src/fourstep.jl:166-180)
template <typename T>
static bool fourstep_split(i64 n, int width, i64 N2in, i64* N1o, i64* N2o) {
  int W = pick_width<T>();
  if (W <= 1) return false;
  i64 S = (i64)width * W;
  i64 N2 = N2in;
  if (N2 == 0) {
    i64 r = isqrt_(n);
    i64 nflat = FS_INNER_MAX / (4 * width * W * (i64)sizeof(T));
    N2 = fs_pick(n, S, std::max(std::min(r, nflat), r / 2));
    if (N2 == 0) return false;
  }
  i64 N1 = n / N2;
  bool ok = N1 * N2 == n && N1 >= S && N2 >= S && factor_radices(N1).ok && factor_radices(N2).ok;
  *N1o = N1; *N2o = N2;
  return ok;
}
template <typename T>
static bool fs_tiled(i64 N1, i64 N2) { return N1 % pick_width<T>() == 0 && N2 % pick_width<T>() == 0; }

// _fs_width (src/fourstep.jl:259-268)
template <typename T>
static int fs_width(i64 N2, i64 N1 = 0) {
  int W = pick_width<T>();
  int w = std::max<i64>(1, (256 + 2 * W * (i64)sizeof(T) - 1) / (2 * W * (i64)sizeof(T)));
  auto fits = [&](int w_) {
    return 4 * (i64)w_ * W * std::max(N1, N2) * (i64)sizeof(T) <= FS_INNER_MAX &&
           (N1 == 0 || (N1 % ((i64)w_ * W) == 0 && N2 % ((i64)w_ * W) == 0));
  };
  while (w > 1 && !fits(w)) w--;
  return w;
}
// _fs_min_bytes / _use_fourstep (src/fourstep.jl:215-226)
template <typename T>
static i64 fs_min_bytes(bool threaded, bool wide) {
  if (!wide) return threaded ? (1 << 20) : (8 << 20);
  if (threaded) return 1 << 19;
  return sizeof(T) >= 8 ? (3 << 20) : (5 << 20);
}
template <typename T>
static bool use_fourstep(i64 n, bool threaded) {
  i64 N1, N2;
  if (!fourstep_split<T>(n, 1, 0, &N1, &N2) || !fs_tiled<T>(N1, N2)) return false;
  bool wide = fs_width<T>(N2, N1) > 1;
  return 2 * n * (i64)sizeof(T) >= fs_min_bytes<T>(threaded, wide);
}
// _use_ragged (src/fourstep.jl:238-247)
template <typename T>
static bool use_ragged(i64 n, bool threaded) {
  i64 a2 = (i64)1 << __builtin_ctzll((unsigned long long)n);
  i64 W4 = 4 * pick_width<T>();
  bool ok = (a2 < W4 && n >= (sizeof(T) >= 8 ? 2048 : 1024)) ||
            (sizeof(T) >= 8 && a2 == W4 && n >= (1 << 14)) || (threaded && n >= (1 << 15));
  if (!ok) return false;
  i64 N1, N2;
  if (!fourstep_split<T>(n, 1, 0, &N1, &N2)) return false;
  return !fs_tiled<T>(N1, N2);
}
// _slow_smooth (src/plan.jl:183-187)
template <typename T>
static bool slow_smooth(i64 n) {
  int a = __builtin_ctzll((unsigned long long)n);
  return sizeof(T) < 8 && (n >> a) > 1 && 48 <= n && n <= 16384 && ((i64)1 << a) < 4 * pick_width<T>();
}

// InnerFourStep (src/fourstep.jl:18-113): a length-N lane transform, nested
// as N = M1*M2 when the lane buffers would outgrow the cache budget.
template <typename T>
struct LaneFFT {
  i64 N, L;
  int D;
  bool nested = false;
  std::vector<Stage<T>> st;    // unnested chain (allow_small = false)
  i64 M1 = 1, M2 = 1;
  std::vector<Stage<T>> stA, stB;
  std::vector<T> twr, twi;     // tw[j1 + M1*k2] = w_N^{j1*k2}
  LaneFFT(i64 N_, i64 L_, int D_) : N(N_), L(L_), D(D_) {
    if (4 * L * N * (i64)sizeof(T) > FS_INNER_MAX) {
      i64 m2 = (i64)1 << (__builtin_ctzll((unsigned long long)N) / 2);
      if (m2 > 1) {
        nested = true;
        M2 = m2; M1 = N / M2;
        stA = build_stages<T>(M2, D, false);
        stB = build_stages<T>(M1, D, false);
        twr.resize(N); twi.resize(N);
        for (i64 k2 = 0; k2 < M2; ++k2)
          for (i64 j1 = 0; j1 < M1; ++j1) {
            double s, c;
            sincospi((double)(2 * D * j1 * k2) / (double)N, &s, &c);
            twr[j1 + M1 * k2] = (T)c; twi[j1 + M1 * k2] = (T)s;
          }
        return;
      }
    }
    st = build_stages<T>(N, D, false);
  }
  // (are, aim): N rows of L lanes (row j at L*j), in natural order; result
  // in natural order in (are, aim). b*, c*: scratch of N*L each.
  void run(T* are, T* aim, T* bre, T* bim, T* cre, T* cim) const {
    if (!nested) {
      bool sw = run_chain(are, aim, bre, bim, st, 0, st.size(), N, 1, L, D, 1);
      if (sw) { std::memcpy(are, bre, sizeof(T) * N * L); std::memcpy(aim, bim, sizeof(T) * N * L); }
      return;
    }
    // first transforms over j2 of rows j1 + M1*j2, twiddle, transform over j1
    for (i64 j1 = 0; j1 < M1; ++j1) {
      for (i64 j2 = 0; j2 < M2; ++j2)
        for (i64 l = 0; l < L; ++l) {
          bre[L * j2 + l] = are[L * (j1 + M1 * j2) + l];
          bim[L * j2 + l] = aim[L * (j1 + M1 * j2) + l];
        }
      bool sw = run_chain(bre, bim, cre, cim, stA, 0, stA.size(), M2, 1, L, D, 1);
      const T* rr = sw ? cre : bre;
      const T* ri = sw ? cim : bim;
      // twiddled rows to slot j1 + M1*k2 (block k2 holds the j1 rows)
      for (i64 k2 = 0; k2 < M2; ++k2) {
        T wr = twr[j1 + M1 * k2], wi = twi[j1 + M1 * k2];
        for (i64 l = 0; l < L; ++l) {
          T yr = rr[L * k2 + l], yi = ri[L * k2 + l];
          tmp_re[(size_t)L * (j1 + M1 * k2) + l] = std::fma(yr, wr, -(yi * wi));
          tmp_im[(size_t)L * (j1 + M1 * k2) + l] = std::fma(yr, wi, yi * wr);
        }
      }
    }
    // transforms over j1 for each k2; output row k = k2 + M2*k1
    for (i64 k2 = 0; k2 < M2; ++k2) {
      T* br = tmp_re.data() + (size_t)L * M1 * k2;
      T* bi = tmp_im.data() + (size_t)L * M1 * k2;
      bool sw = run_chain(br, bi, bre, bim, stB, 0, stB.size(), M1, 1, L, D, 1);
      const T* rr = sw ? bre : br;
      const T* ri = sw ? bim : bi;
      for (i64 k1 = 0; k1 < M1; ++k1)
        for (i64 l = 0; l < L; ++l) {
          are[L * (k2 + M2 * k1) + l] = rr[L * k1 + l];
          aim[L * (k2 + M2 * k1) + l] = ri[L * k1 + l];
        }
    }
  }
  mutable std::vector<T> tmp_re, tmp_im;
  void alloc_tmp() const {
    if (nested) { tmp_re.resize((size_t)N * L); tmp_im.resize((size_t)N * L); }
  }
};

// FourStepPlan (src/fourstep.jl:130-156, 272-330, 338-495).
template <typename T>
struct FourStepPlan : PlanBase {
  int D;
  T scale;
  i64 N1, N2, S, G, Z1, R, K;
  std::vector<T> b1r, b1i, b2r, b2i, hir, hii, lor, loi;
  std::vector<T> zre, zim;
  std::vector<std::unique_ptr<LaneFFT<T>>> innerA, innerB;  // per task
  std::vector<std::vector<T>> bufs;                          // per task, 6 planes
  i64 nb;
  int nt;
  FourStepPlan(i64 n_, int D_, T scale_, int nthreads, i64 N2req = 0, int width = 0) : D(D_), scale(scale_) {
    n = n_;
    route = ORC_FOURSTEP;
    int W = pick_width<T>();
    if (!fourstep_split<T>(n, std::max(width, 1), N2req, &N1, &N2))
      throw std::runtime_error("no four-step split");
    if (width == 0) width = fs_width<T>(N2, N1);
    S = G = (i64)width * W;
    i64 zpad = S;
    auto om = [&](i64 e, T* c, T* s) {
      double ss, cc;
      sincospi((double)(2 * D * e) / (double)n, &ss, &cc);
      *c = (T)cc; *s = (T)ss;
    };
    R = (i64)1 << (__builtin_ctzll((unsigned long long)N2) / 2);
    i64 ntt = (N2 + R - 1) / R;
    b1r.resize(S * R); b1i.resize(S * R); b2r.resize(S * ntt); b2i.resize(S * ntt);
    for (i64 r = 0; r < R; ++r)
      for (i64 l = 0; l < S; ++l) om(r * l, &b1r[S * r + l], &b1i[S * r + l]);
    for (i64 t = 0; t < ntt; ++t)
      for (i64 l = 0; l < S; ++l) om(R * t * l, &b2r[S * t + l], &b2i[S * t + l]);
    K = isqrt_(n - 1) + 1;
    i64 nh = (n + K - 1) / K;
    hir.resize(nh); hii.resize(nh); lor.resize(K); loi.resize(K);
    for (i64 i = 0; i < nh; ++i) om(i * K, &hir[i], &hii[i]);
    for (i64 i = 0; i < K; ++i) om(i, &lor[i], &loi[i]);
    Z1 = N1 + zpad;
    i64 na = (N1 + S - 1) / S, ng = (N2 + G - 1) / G;
    nt = (int)std::min<i64>(std::min<i64>(std::max(nthreads, 1), na),
                            std::min<i64>(ng, std::max<i64>(1, n / FS_TASK_MIN)));
    for (int i = 0; i < nt; ++i) {
      innerA.emplace_back(new LaneFFT<T>(N2, S, D));
      innerB.emplace_back(new LaneFFT<T>(N1, G, D));
      innerA.back()->alloc_tmp();
      innerB.back()->alloc_tmp();
    }
    nb = std::max(S * N2, G * N1);
    bufs.resize(nt);
    for (auto& b : bufs) b.assign(6 * nb, (T)0);
    i64 nz = Z1 * ng * G;
    zre.assign(nz, (T)0); zim.assign(nz, (T)0);
  }
  // pass A, strips [slo, shi) (src/fourstep.jl:364-428)
  void pass_a(int ci, const T* x, i64 slo, i64 shi) {
    T* are = bufs[ci].data();
    T* aim = are + nb;
    T* bre = aim + nb;
    T* bim = bre + nb;
    T* cre = bim + nb;
    T* cim = cre + nb;
    for (i64 sidx = slo; sidx < shi; ++sidx) {
      i64 c = S * sidx;
      i64 lim = N1 - c;
      for (i64 j2 = 0; j2 < N2; ++j2)
        for (i64 l = 0; l < S; ++l) {
          if (l < lim) {
            i64 e = c + N1 * j2 + l;
            are[S * j2 + l] = x[2 * e]; aim[S * j2 + l] = x[2 * e + 1];
          } else {
            are[S * j2 + l] = 0; aim[S * j2 + l] = 0;
          }
        }
      innerA[ci]->run(are, aim, bre, bim, cre, cim);
      for (i64 k2 = 0; k2 < N2; ++k2) {
        i64 e = c * k2, hi = e / K, lo = e % K;
        T ar = hir[hi] * lor[lo] - hii[hi] * loi[lo];
        T ai = hir[hi] * loi[lo] + hii[hi] * lor[lo];
        i64 tt = k2 / R, rr = k2 % R;
        for (i64 l = 0; l < S; ++l) {
          T b1rv = b1r[S * rr + l], b1iv = b1i[S * rr + l], b2rv = b2r[S * tt + l], b2iv = b2i[S * tt + l];
          T br = std::fma(b1rv, b2rv, -(b1iv * b2iv));
          T bi = std::fma(b1rv, b2iv, b1iv * b2rv);
          T twr = std::fma(ar, br, -(ai * bi));
          T twi = std::fma(ar, bi, ai * br);
          T yr = are[S * k2 + l], yi = aim[S * k2 + l];
          zre[c + Z1 * k2 + l] = std::fma(yr, twr, -(yi * twi));
          zim[c + Z1 * k2 + l] = std::fma(yr, twi, yi * twr);
        }
      }
    }
  }
  // pass B, groups [glo, ghi) (src/fourstep.jl:433-495)
  void pass_b(int ci, T* y, i64 glo, i64 ghi) {
    T* are = bufs[ci].data();
    T* aim = are + nb;
    T* bre = aim + nb;
    T* bim = bre + nb;
    T* cre = bim + nb;
    T* cim = cre + nb;
    for (i64 gidx = glo; gidx < ghi; ++gidx) {
      i64 c2 = G * gidx;
      i64 lim = N2 - c2;
      for (i64 g = 0; g < G; ++g) {
        i64 off = Z1 * (c2 + g);
        for (i64 j1 = 0; j1 < N1; ++j1) { are[G * j1 + g] = zre[off + j1]; aim[G * j1 + g] = zim[off + j1]; }
      }
      innerB[ci]->run(are, aim, bre, bim, cre, cim);
      for (i64 k1 = 0; k1 < N1; ++k1)
        for (i64 g = 0; g < G && g < lim; ++g) {
          i64 e = c2 + N2 * k1 + g;
          y[2 * e] = are[G * k1 + g] * scale;
          y[2 * e + 1] = aim[G * k1 + g] * scale;
        }
    }
  }
  void exec(const void* xv, void* yv) override {
    const T* x = (const T*)xv;
    T* y = (T*)yv;
    i64 na = (N1 + S - 1) / S, ng = (N2 + G - 1) / G;
    if (nt > 1) {
      tforeach_chunks(na, nt, 1, [&](int ci, i64 lo, i64 hi) { pass_a(ci, x, lo, hi); });
      tforeach_chunks(ng, nt, 1, [&](int ci, i64 lo, i64 hi) { pass_b(ci, y, lo, hi); });
    } else {
      pass_a(0, x, 0, na);
      pass_b(0, y, 0, ng);
    }
  }
  void info(std::vector<i64>& v) override {
    v.push_back(route); v.push_back(n); v.push_back(N1); v.push_back(N2); v.push_back(S);
    v.push_back(innerA[0]->nested); v.push_back(innerB[0]->nested);
  }
};

// ---- resampling (src/resample.jl) -----------------------------------------
static const int SMOOTH_ODD[7] = {1, 3, 5, 7, 9, 15, 21};
static int top_set_bit(i64 x) { return x <= 0 ? 0 : 64 - __builtin_clzll((unsigned long long)x); }
static i64 nextsmooth(i64 N) {  // src/resample.jl:13-21
  i64 best = INT64_MAX;
  for (int o : SMOOTH_ODD) {
    int k = std::max(6, top_set_bit((N + o - 1) / o - 1));
    i64 c = (i64)o << k;
    if (c < best) best = c;
  }
  return best;
}
static i64 nextsmooth7(i64 N) {  // src/resample.jl:25-31
  i64 m = N;
  while (!factor_smooth(m)) m++;
  return m;
}
// _gausslegendre (src/resample.jl:33-53)
static void gausslegendre(int nq, std::vector<double>& z, std::vector<double>& wq) {
  z.assign(nq, 0); wq.assign(nq, 0);
  const double eps = 2.220446049250313e-16;
  for (int i = 1; i <= nq; ++i) {
    double x = cospi_((i - 0.25) / (nq + 0.5));
    double dp = 1;
    for (int it = 0; it < 20; ++it) {
      double p0 = 1, p1 = x;
      for (int k = 2; k <= nq; ++k) {
        double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1; p1 = p2;
      }
      dp = nq * (x * p1 - p0) / (x * x - 1);
      double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 4 * eps) break;
    }
    z[i - 1] = x;
    wq[i - 1] = 2 / ((1 - x * x) * dp * dp);
  }
}
static inline double es_(double z, double beta) {  // src/resample.jl:55
  return std::fabs(z) >= 1 ? 0.0 : std::exp(beta * (std::sqrt(1 - z * z) - 1));
}

// _fit_weights_d (src/resample.jl:137-169): degree-d Chebyshev interpolants
// of every tap's weight on each of P pieces of the offset, converted to
// monomials in the local variable t in [-1, 1] and rounded to T; returns the
// largest error of the rounded polynomials on 4d + 4 points.
template <typename T>
static double fit_weights_d(double beta, i64 w, i64 P, int d, std::vector<T>& C) {
  const i64 h = w / 2;
  std::vector<double> tj(d + 1), fj(d + 1), mono(d + 1), Tkm(d + 1), Tk(d + 1), Tn(d + 1);
  for (int j = 0; j <= d; ++j) tj[j] = cospi_((j + 0.5) / (double)(d + 1));
  C.assign((size_t)(P * (d + 1) * w), (T)0);
  double err = 0;
  for (i64 p = 0; p < P; ++p)
    for (i64 i = 0; i < w; ++i) {
      auto f = [&](double t) { return es_((((double)p + (t + 1) / 2) / (double)P + h - 1 - i) / (double)h, beta); };
      for (int j = 0; j <= d; ++j) fj[j] = f(tj[j]);
      std::fill(mono.begin(), mono.end(), 0.0);
      std::fill(Tkm.begin(), Tkm.end(), 0.0);
      std::fill(Tk.begin(), Tk.end(), 0.0);
      Tkm[0] = 1;  // T_0, T_1 in monomials
      Tk[1] = 1;
      for (int k = 0; k <= d; ++k) {
        double a = 0;
        for (int j = 0; j <= d; ++j) {
          const double term = fj[j] * cospi_((double)k * (j + 0.5) / (double)(d + 1));
          a = j == 0 ? term : a + term;
        }
        a = a * 2 / (double)(d + 1);
        if (k == 0) a /= 2;
        const std::vector<double>& Tc = k == 0 ? Tkm : Tk;
        for (int c = 0; c <= d; ++c) mono[c] = mono[c] + a * Tc[c];
        if (k >= 1) {  // T_{k+1} = 2t T_k - T_{k-1}
          for (int c = 0; c <= d; ++c) Tn[c] = -Tkm[c];
          for (int c = 1; c <= d; ++c) Tn[c] = Tn[c] + 2 * Tk[c - 1];
          Tkm.swap(Tk);
          Tk.swap(Tn);
        }
      }
      for (int c = 0; c <= d; ++c) {
        const T v = (T)mono[c];
        C[(size_t)((p * (d + 1) + c) * w + i)] = v;
        mono[c] = (double)v;
      }
      const int ns = 4 * d + 4;
      for (int q = 0; q < ns; ++q) {
        const double t = -1.0 + 2.0 * (double)q / (double)(ns - 1);
        double ev = mono[d];  // evalpoly (Horner)
        for (int c = d - 1; c >= 0; --c) ev = std::fma(t, ev, mono[c]);
        err = std::max(err, std::fabs(ev - f(t)));
      }
    }
  return err;
}
// _fit_weights (src/resample.jl:126-135): the degree grows until the fit
// error is <= tolw or stops halving
template <typename T>
static int fit_weights(double beta, i64 w, i64 P, double tolw, std::vector<T>& C) {
  std::vector<T> prev, cur;
  double preverr = fit_weights_d<T>(beta, w, P, 1, prev);
  for (int d = 2; d <= 30; ++d) {
    const double err = fit_weights_d<T>(beta, w, P, d, cur);
    if (err <= tolw) { C.swap(cur); return d; }
    if (err > preverr / 2) { C.swap(prev); return d - 1; }
    prev.swap(cur);
    preverr = err;
  }
  C.swap(prev);
  return 30;
}

static const i64 RS_TABLE_MAX = 1 << 21;  // _RS_TABLE_MAX (src/resample.jl:173)

// Plan-independent resampling parts (src/resample.jl:202-256): a weight
// table, or -- for a 1-D plan whose table would exceed RS_TABLE_MAX --
// piecewise polynomial weights (WPoly, src/resample.jl:62-118).
template <typename T>
struct RsParts {
  i64 n, m, w, h;
  double beta;
  std::vector<T> corr, wt;
  std::vector<int32_t> l0;
  bool poly = false;
  int deg = 0;
  i64 P = 0;
  std::vector<T> C;  // C[(p (deg + 1) + c) w + i]: coefficient c of tap i, piece p
  RsParts(i64 n_, int D, T scale, i64 m_ = 0, bool allow_poly = false) : n(n_) {
    (void)D;
    const double epsT = sizeof(T) >= 8 ? 2.220446049250313e-16 : 1.1920928955078125e-07;
    double tol = 10 * epsT;
    m = m_ ? m_ : nextsmooth((i64)std::ceil(2.0 * n));
    double ratio = std::max((double)n / m, 0.5);
    i64 wc = (i64)std::ceil(std::log(1 / tol) / (M_PI * std::sqrt(1 - ratio)));
    w = 4 * ((wc + 3) / 4);
    beta = 0.97 * M_PI * w * (1 - (double)n / (2.0 * m));
    h = w / 2;
    std::vector<double> zq, wq;
    gausslegendre((int)(2 * w + 20), zq, wq);
    corr.resize(n);
    i64 hp = (n + 1) / 2;
    for (i64 j = 0; j < n; ++j) {
      i64 jp = j < hp ? j : j - n;
      double nu = (double)jp / m;
      double Phi = 0;
      for (size_t q = 0; q < zq.size(); ++q) {
        if (!(zq[q] > 0)) continue;
        Phi += wq[q] * es_(zq[q], beta) * cospi_(nu * w * zq[q]);
      }
      corr[j] = (T)((double)scale / (w * Phi));
    }
    l0.resize(n);
    for (i64 k = 0; k < n; ++k) {
      __int128 km = (__int128)k * m;
      l0[k] = (int32_t)((i64)(km / n) - h + 1);
    }
    poly = allow_poly && n * w * (i64)sizeof(T) > RS_TABLE_MAX;
    if (poly) {
      P = sizeof(T) >= 8 ? 32 : 64;
      deg = fit_weights<T>(beta, w, P, tol / 16, C);
      return;
    }
    wt.resize(n * w);
    for (i64 k = 0; k < n; ++k) {
      __int128 km = (__int128)k * m;
      i64 r = (i64)(km % n);
      double delta = (double)r / n;
      for (i64 i = 0; i < w; ++i) wt[k * w + i] = (T)es_((delta + h - 1 - i) / h, beta);
    }
  }
  // the w weights of output k (_wget: a table row, or Horner across the
  // taps in t = 2 (s - piece) - 1, s = (k m mod n) P / n)
  const T* weights(i64 k, T* buf) const {
    if (!poly) return &wt[k * w];
    const i64 r = (i64)(((__int128)k * m) % n);
    const double sp = (double)r * ((double)P / (double)n);
    const i64 pc = std::min((i64)sp, P - 1);
    const T t = (T)(2 * (sp - (double)pc) - 1);
    const size_t base = (size_t)(pc * (deg + 1));
    for (i64 i = 0; i < w; ++i) {
      T v = C[(base + deg) * w + i];
      for (int c = deg - 1; c >= 0; --c) v = std::fma(v, t, C[(base + c) * w + i]);
      buf[i] = v;
    }
    return buf;
  }
};

// ResamplePlan (src/resample.jl:175-194, 258-276, 392-424).
template <typename T>
struct ResamplePlan : PlanBase {
  int D;
  T scale;
  RsParts<T> parts;
  std::unique_ptr<FFTPlan<T>> p;
  ResamplePlan(i64 n_, int D_, T scale_) : D(D_), scale(scale_), parts(n_, D_, scale_, 0, true) {
    n = n_;
    route = ORC_RESAMPLE;
    p.reset(new FFTPlan<T>(parts.m, D, (T)1, 1));
  }
  void exec(const void* xv, void* yv) override {
    const T* x = (const T*)xv;
    T* y = (T*)yv;
    i64 m = parts.m, hp = (n + 1) / 2;
    T* are = p->are.data();
    T* aim = p->aim.data();
    // _deconv! x2 (src/resample.jl:281-301) and zero fill
    for (i64 c = 0; c < hp; ++c) { are[c] = x[2 * c] * parts.corr[c]; aim[c] = x[2 * c + 1] * parts.corr[c]; }
    for (i64 c = 0; c < n - hp; ++c) {
      i64 j = hp + c;
      are[m - n + hp + c] = x[2 * j] * parts.corr[j];
      aim[m - n + hp + c] = x[2 * j + 1] * parts.corr[j];
    }
    for (i64 j = hp; j < m - n + hp; ++j) { are[j] = 0; aim[j] = 0; }
    bool sw = run_chain(are, aim, p->bre.data(), p->bim.data(), p->stages, 0, p->stages.size(), m, 1, 1, D, 1);
    const T* gre = sw ? p->bre.data() : are;
    const T* gim = sw ? p->bim.data() : aim;
    // _interp! (src/resample.jl:392-424): blocks of V/2 outputs whose
    // windows lie inside the grid sum as _interp_block! does, the others
    // tap by tap (the ordered sum of a vector)
    const i64 w = parts.w, V = pick_width<T>();
    const i64 sl = std::min(w, V);
    const bool blockable = V > 1 && (w % V == 0 || V % w == 0) && (sl & (sl - 1)) == 0;  // _blockable
    const i64 Bk = blockable ? V / 2 : 0;
    std::vector<T> pr(w), cs(sl), wbuf(w);
    // _chunksum to sl lanes (chunks added left to right), then the tree
    // halving of _tree_reduce_code: lane j += lane j + L/2
    auto block_dot = [&](const T* g, i64 lk, const T* wv) {
      for (i64 i = 0; i < w; ++i) pr[i] = g[lk + i] * wv[i];
      for (i64 j = 0; j < sl; ++j) {
        T c = pr[j];
        for (i64 ch = 1; ch < w / sl; ++ch) c = c + pr[ch * sl + j];
        cs[j] = c;
      }
      for (i64 L = sl; L > 1; L /= 2)
        for (i64 j = 0; j < L / 2; ++j) cs[j] = cs[j] + cs[j + L / 2];
      return cs[0];
    };
    // _wblock_ok: the table's windows, or (polynomial weights) a bound from
    // the block's first grid row and floor((B - 1) m / n) + 1 rows on
    auto block_ok = [&](i64 k) {
      if (!parts.poly) return parts.l0[k] >= 0 && parts.l0[k + Bk - 1] + w <= m;
      const i64 q = (i64)(((__int128)k * m) / n);
      const i64 g = (i64)(((__int128)(Bk - 1) * m) / n);
      return q - parts.h + 1 >= 0 && q + g + 1 - parts.h + 1 + w <= m;
    };
    i64 k = 0;
    while (k < n) {
      if (Bk > 0 && k + Bk <= n && block_ok(k)) {
        for (i64 j = 0; j < Bk; ++j) {
          const T* wv = parts.weights(k + j, wbuf.data());
          const T re = block_dot(gre, parts.l0[k + j], wv);
          const T im = block_dot(gim, parts.l0[k + j], wv);
          y[2 * (k + j)] = re; y[2 * (k + j) + 1] = im;
        }
        k += Bk;
        continue;
      }
      i64 lk = parts.l0[k];
      const T* wv = parts.weights(k, wbuf.data());
      T re = 0, im = 0;
      for (i64 i = 0; i < w; ++i) {
        i64 l = lk + i;
        l %= m;
        if (l < 0) l += m;
        re += wv[i] * gre[l];
        im += wv[i] * gim[l];
      }
      y[2 * k] = re; y[2 * k + 1] = im;
      ++k;
    }
  }
  void info(std::vector<i64>& v) override {  // route, n, m, w, polynomial weight degree (0: table)
    v.push_back(route); v.push_back(n); v.push_back(parts.m); v.push_back(parts.w);
    v.push_back(parts.poly ? parts.deg : 0);
  }
};

// _anyplan routing (src/plan.jl:192-206), defined after the plans for
// non-smooth lengths below
template <typename T>
static PlanBase* anyplan(i64 n, int D, T scale, int nthreads);

// ---- real transforms (src/real.jl) ----------------------------------------
template <typename T>
struct RfftPlan {
  i64 n;
  std::unique_ptr<PlanBase> inner;
  std::vector<T> twr, twi, buf, buf2;
  RfftPlan(i64 n_, int nthreads) : n(n_) {
    bool even = n % 2 == 0;
    i64 len = even ? n / 2 : n;
    inner.reset(anyplan<T>(len, -1, (T)1, nthreads));
    if (even) {
      twr.resize(len + 1); twi.resize(len + 1);
      for (i64 k = 0; k <= len; ++k) {  // real_twiddles (src/real.jl:26-39)
        double s, c;
        sincospi(-1 * ((double)(2 * k) / n), &s, &c);
        twr[k] = (T)c; twi[k] = (T)s;
      }
    }
    buf.resize(2 * len);
    buf2.resize(even ? 0 : 2 * n);
  }
  void exec(const T* x, T* y) {  // src/real.jl:80-142
    if (n % 2 == 0) {
      i64 h = n / 2;
      inner->exec(x, buf.data());
      const T* Z = buf.data();
      y[0] = Z[0] + Z[1]; y[1] = 0;
      y[2 * h] = Z[0] - Z[1]; y[2 * h + 1] = 0;
      const T half = (T)0.5;
      for (i64 k = 1; k < h; ++k) {
        T ar = Z[2 * k], ai = Z[2 * k + 1];
        T br = Z[2 * (h - k)], bi = -Z[2 * (h - k) + 1];
        T xer = (ar + br) * half, xei = (ai + bi) * half;
        T xor_ = (ar - br) * half, xoi = (ai - bi) * half;
        T wr = twr[k], wi = twi[k];
        y[2 * k] = xer + std::fma(wr, xoi, wi * xor_);
        y[2 * k + 1] = xei + std::fma(wi, xoi, -(wr * xor_));
      }
    } else {
      for (i64 j = 0; j < n; ++j) { buf[2 * j] = x[j]; buf[2 * j + 1] = 0; }
      inner->exec(buf.data(), buf2.data());
      std::memcpy(y, buf2.data(), sizeof(T) * 2 * (n / 2 + 1));
    }
  }
};

template <typename T>
struct IrfftPlan {
  i64 n;
  T pre;
  std::unique_ptr<PlanBase> inner;
  std::vector<T> twr, twi, buf, buf2;
  IrfftPlan(i64 n_, bool normalized, int nthreads) : n(n_) {
    pre = normalized ? (T)0.5 : (T)1;
    bool even = n % 2 == 0;
    i64 len = even ? n / 2 : n;
    inner.reset(anyplan<T>(len, +1, normalized ? default_scale<T>(len, +1) : (T)1, nthreads));
    if (even) {
      twr.resize(len); twi.resize(len);
      for (i64 k = 0; k < len; ++k) {
        double s, c;
        sincospi(+1 * ((double)(2 * k) / n), &s, &c);
        twr[k] = (T)c; twi[k] = (T)s;
      }
    }
    buf.resize(2 * len);
    buf2.resize(even ? 0 : 2 * n);
  }
  void exec(const T* X, T* y) {  // src/real.jl:144-211
    if (n % 2 == 0) {
      i64 h = n / 2;
      T* Z = buf.data();
      for (i64 k = 0; k < h; ++k) {
        T ar = X[2 * k], ai = X[2 * k + 1];
        T br = X[2 * (h - k)], bi = -X[2 * (h - k) + 1];
        T xer = (ar + br) * pre, xei = (ai + bi) * pre;
        T xdr = (ar - br) * pre, xdi = (ai - bi) * pre;
        T wr = twr[k], wi = twi[k];
        T tr = std::fma(wr, xdr, -(wi * xdi));
        T ti = std::fma(wr, xdi, wi * xdr);
        Z[2 * k] = xer - ti;
        Z[2 * k + 1] = xei + tr;
      }
      inner->exec(Z, y);
    } else {
      i64 h = n / 2;
      T* b = buf.data();
      for (i64 k = 0; k <= h; ++k) { b[2 * k] = X[2 * k]; b[2 * k + 1] = X[2 * k + 1]; }
      for (i64 k = 1; k <= h; ++k) { b[2 * (n - k)] = X[2 * k]; b[2 * (n - k) + 1] = -X[2 * k + 1]; }
      inner->exec(b, buf2.data());
      for (i64 j = 0; j < n; ++j) y[j] = buf2[2 * j];
    }
  }
};

// ---- N-d (src/ndplan.jl) ---------------------------------------------------
// Batched resampling along one dim (RsPass, src/resample.jl:434-588).
template <typename T>
struct RsPass {
  i64 n, m, w, B;
  RsParts<T> parts;
  std::vector<Stage<T>> stages;
  RsPass(i64 n_, int D, i64 B_) : n(n_), B(B_), parts(n_, D, (T)1, nextsmooth7(2 * n_)) {
    m = parts.m; w = parts.w;
    stages = build_stages<T>(m, D, B == 1);
  }
  // rows of B lanes at xre/xim + off (row j lane i at off + B*j + i), in
  // place. load(j, i, c, xr, xi, &yr, &yi), when given, replaces the
  // deconvolution x c of row j, lane i (CompositePlan folds its twiddles in).
  template <class Load>
  void run(T* xre, T* xim, i64 off, int D, Load load) {
    std::vector<T> pre(m * B), pim(m * B), qre(m * B), qim(m * B);
    i64 hp = (n + 1) / 2;
    for (i64 j = 0; j < n; ++j) {
      i64 jj = j < hp ? j : m - n + j;
      T c = parts.corr[j];
      for (i64 i = 0; i < B; ++i) load(j, i, c, xre[off + B * j + i], xim[off + B * j + i], &pre[B * jj + i], &pim[B * jj + i]);
    }
    for (i64 j = hp; j < m - n + hp; ++j)
      for (i64 i = 0; i < B; ++i) { pre[B * j + i] = 0; pim[B * j + i] = 0; }
    bool sw = run_chain(pre.data(), pim.data(), qre.data(), qim.data(), stages, 0, stages.size(), m, 1, B, D, 1);
    const T* gre = sw ? qre.data() : pre.data();
    const T* gim = sw ? qim.data() : pim.data();
    for (i64 k = 0; k < n; ++k) {
      i64 l = parts.l0[k];
      for (i64 i = 0; i < B; ++i) {
        T ar = 0, ai = 0;
        for (i64 t = 0; t < w; ++t) {
          i64 g = l + t;
          if (g < 0) g += m;
          if (g >= m) g -= m;
          ar = std::fma(parts.wt[w * k + t], gre[B * g + i], ar);
          ai = std::fma(parts.wt[w * k + t], gim[B * g + i], ai);
        }
        xre[off + B * k + i] = ar;
        xim[off + B * k + i] = ai;
      }
    }
  }
  void run(T* xre, T* xim, i64 off, int D) {
    run(xre, xim, off, D, [](i64, i64, T c, T xr, T xi, T* yr, T* yi) { *yr = xr * c; *yi = xi * c; });
  }
};

// ---- Gaussian resampling: HvdhPlan (src/hvdh.jl) ----------------------------
// Restated with the reference's own evaluation of the Gaussian entries: the
// band's columns and the spread's weights advance by multiplicative
// recurrences seeded exactly (by its polynomial exp, _vexp) every few
// columns / vectors, lane by lane as its SIMD code runs them
// (src/hvdh.jl:99-114, 337-470, 472-540). The batched pass along a strided
// axis (HvPass, src/hvdh.jl:690-760) tabulates its spread weights with the
// library exp instead, factors one cyclic chunk, and transforms with the
// no-small chain; HvdhPlan's pass form restates that.
static i64 gcd_i(i64 a, i64 b) {
  a = a < 0 ? -a : a; b = b < 0 ? -b : b;
  while (b) { i64 t = a % b; a = b; b = t; }
  return a;
}
static i64 invmod_i(i64 a, i64 m) {  // a^{-1} mod m, gcd(a, m) = 1
  i64 g = m, x = 0, x1 = 1, aa = ((a % m) + m) % m;
  while (aa) {
    i64 q = g / aa, t = g - q * aa;
    g = aa; aa = t;
    t = x - q * x1; x = x1; x1 = t;
  }
  return ((x % m) + m) % m;
}
static i64 fld_i(i64 a, i64 b) { i64 q = a / b; if ((a % b != 0) && ((a < 0) != (b < 0))) q--; return q; }
static i64 cld_i(i64 a, i64 b) { return -fld_i(-a, b); }
static i64 mod_i(i64 a, i64 m) { i64 r = a % m; return r < 0 ? r + m : r; }

// _vexp (src/hvdh.jl:99-114): exp for |x| <~ 10 by Cody-Waite reduction by
// ln 2 (hi + lo split) and a Taylor polynomial in Horner form, 14 terms for
// Float64 and 8 for Float32, scaled by 2^k built from the exponent bits.
static double fact_inv(int j) {  // 1 / j!, j! exact in a double for j <= 13
  double f = 1;
  for (int i = 2; i <= j; ++i) f *= i;
  return 1.0 / f;
}
template <typename T>
static T vexp(T x);
template <>
inline double vexp<double>(double x) {
  static const struct C { double c[14]; C() { for (int j = 0; j < 14; ++j) c[j] = fact_inv(j); } } k;
  const double kf = std::nearbyint(x * 1.4426950408889634);
  double r = std::fma(kf, -6.93147180369123816490e-01, x);
  r = std::fma(kf, -1.90821492927058770002e-10, r);
  double p = k.c[13];
  for (int j = 12; j >= 0; --j) p = std::fma(p, r, k.c[j]);
  const uint64_t bits = (uint64_t)((int64_t)kf + 1023) << 52;
  double sc;
  std::memcpy(&sc, &bits, sizeof sc);
  return p * sc;
}
template <>
inline float vexp<float>(float x) {
  static const struct C { float c[8]; C() { for (int j = 0; j < 8; ++j) c[j] = (float)fact_inv(j); } } k;
  const float kf = std::nearbyint(x * (float)1.4426950408889634);
  float r = std::fma(kf, -(float)0.693145751953125, x);
  r = std::fma(kf, -(float)1.428606765330187045e-6, r);
  float p = k.c[7];
  for (int j = 6; j >= 0; --j) p = std::fma(p, r, k.c[j]);
  const uint32_t bits = (uint32_t)((int32_t)kf + 127) << 23;
  float sc;
  std::memcpy(&sc, &bits, sizeof sc);
  return p * sc;
}

static const double HVDH_THETA_MIN = 1.0 / 128;  // src/hvdh.jl:67
static const i64 HVDH_LTARGET = 256;             // src/hvdh.jl:68
static const i64 HVDH_TABLE_MAX = 8 << 20;       // src/hvdh.jl:75

// _hvdh_t (src/hvdh.jl:78-92): t coprime to n; 0 when there is none
static i64 hvdh_t(i64 n) {
  const i64 N = (i64)std::ceil(n * (1 + HVDH_THETA_MIN));
  i64 t = INT64_MAX;
  if (n % 2 == 1) {
    for (int o : SMOOTH_ODD)
      if (gcd_i(o, n) == 1) t = std::min<i64>(t, (i64)o << top_set_bit((N + o - 1) / o - 1));
  } else {
    for (i64 m = N | 1; m <= 2 * n - 1; m += 2)
      if (factor_smooth(m) && gcd_i(m, n) == 1) { t = m; break; }
  }
  return (t != INT64_MAX && t - n < n) ? t : 0;
}
template <typename T>
static bool use_hvdh(i64 n) { return n % 2 == 1 && n >= (sizeof(T) >= 8 ? 1000 : 16384); }  // src/hvdh.jl:97

// Dense solve A x = b with partial pivoting (Julia's `\` on a square matrix).
static void dense_solve(std::vector<double>& A, std::vector<double>& b, i64 m) {
  for (i64 k = 0; k < m; ++k) {
    i64 p = k;
    for (i64 i = k + 1; i < m; ++i)
      if (std::fabs(A[i * m + k]) > std::fabs(A[p * m + k])) p = i;
    if (p != k) {
      for (i64 j = 0; j < m; ++j) std::swap(A[k * m + j], A[p * m + j]);
      std::swap(b[k], b[p]);
    }
    const double piv = A[k * m + k];
    for (i64 i = k + 1; i < m; ++i) {
      const double f = A[i * m + k] / piv;
      if (f == 0) continue;
      for (i64 j = k; j < m; ++j) A[i * m + j] -= f * A[k * m + j];
      b[i] -= f * b[k];
    }
  }
  for (i64 k = m - 1; k >= 0; --k) {
    double s = b[k];
    for (i64 j = k + 1; j < m; ++j) s -= A[k * m + j] * b[j];
    b[k] = s / A[k * m + k];
  }
}

// _hvdh_halo (src/hvdh.jl:117-145): halo rows from a few dense probes of the
// l-indexed system's inverse
static i64 hvdh_halo(i64 n, i64 t, double a, i64 B, double tol) {
  const double rho = (double)t / n;
  const i64 c = invmod_i(t - n, n);
  std::vector<i64> probes;
  const i64 L = std::min<i64>(n, 16);
  for (i64 k = 0; k < L; ++k)
    probes.push_back(L == 1 ? 0 : (i64)std::nearbyint((double)k * (double)(n - 1) / (double)(L - 1)));
  for (i64 h : {n / 2, n / 2 + 1}) probes.push_back(mod_i(h * c, n));
  i64 P = 64;
  for (;;) {
    i64 H = 0;
    const i64 m = 2 * P + 1;
    for (i64 l0 : probes) {
      // transpose(M) r = e, built transposed: A[j][i] = M[i][j]
      std::vector<double> A(m * m, 0.0), r(m, 0.0);
      for (i64 i = 0; i < m; ++i)
        for (i64 j = std::max<i64>(0, i - B - 1); j <= std::min<i64>(m - 1, i + B + 1); ++j) {
          const i64 li = l0 - P + i, lj = l0 - P + j;
          const double d = rho * lj - (double)fld_i(2 * t * li + n, 2 * n);
          A[j * m + i] = std::exp(-a * d * d);
        }
      r[P] = 1;
      dense_solve(A, r, m);
      double mx = 0;
      for (i64 j = 0; j < m; ++j) mx = std::max(mx, std::fabs(r[j]));
      for (i64 j = 0; j < m; ++j)
        if (std::fabs(r[j]) > tol * mx) H = std::max<i64>(H, std::llabs(j - P));
    }
    if (H < P - 2 * B) return (i64)std::ceil(rho * H) + B;
    P *= 2;
    if (P > 8192) throw std::runtime_error("HvdH halo did not converge");
  }
}

// 2 t l' - 2 n q + n and l' for the first unknown l' with rho l' >= q - 1/2
// (_hvdh_e, src/hvdh.jl:147-151)
static void hvdh_e(i64 n, i64 t, i64 q, i64* e, i64* l) {
  *l = cld_i(2 * n * q - n, 2 * t);
  *e = 2 * t * (*l) - 2 * n * q + n;
}

// HvdhPlan (src/hvdh.jl:30-58, 153-230): scatter, Gaussian spread onto the
// t-grid, length-t transform, banded solve by chunks (K chunks per group,
// L core rows + H halo rows per side), scale n/t. The pass form is the
// batched HvPass's arithmetic for one lane (_hv_parts / _hv_chunk!,
// src/hvdh.jl:727-836): K = 1 and one cyclic chunk (G = 1, L = t),
// tabulated spread weights accumulated tap by tap, the length-t chain
// without the small-stride layout, output scale T(n/t).
template <typename T>
struct HvdhPlan : PlanBase {
  int D;
  T scale;
  bool pass_form;
  i64 t, Delta, c, h, w, B, H, K, G, L, R, rsm;
  double alpha, a, b;
  T aT, dT;                  // T(a), T(Delta/n): the column seeds' arguments
  T rc[7];                   // column-recurrence factors (_hvdh_step)
  std::vector<T> chT;        // ch[d] = exp(-a d^2), d = 1..B
  std::vector<i64> se, sx, so;
  std::unique_ptr<PlanBase> pt;
  std::vector<Stage<T>> tstages;  // pass form: the length-t chain
  bool tab;  // factors precomputed (:table) or rebuilt per call (:fly)
  // per chunk: multipliers f[i][k] (k = 1..B), 1/U_ii, U_{i,i+1..i+B}, output index
  std::vector<T> lt, ut;
  std::vector<i64> ot;
  static const i64 kReseed = 4;   // _HVDH_RESEED (src/hvdh.jl:70)
  static const i64 kSReseed = 8;  // _HVDH_SRESEED (src/hvdh.jl:72)
  static const i64 kJ = 8;        // spread rows per block (_hvdh_spread!'s J)
  // factors: 0 :auto, 1 :table, 2 :fly (src/hvdh.jl:187-191)
  HvdhPlan(i64 n_, int D_, T scale_, int factors, bool pass = false) : D(D_), scale(scale_), pass_form(pass) {
    n = n_;
    route = ORC_HVDH;
    t = hvdh_t(n);
    if (!t) throw std::invalid_argument("no coprime smooth t");
    Delta = t - n;
    c = invmod_i(Delta, n);
    alpha = sizeof(T) >= 8 ? 1.45 : 1.0;  // _hvdh_alpha (src/hvdh.jl:64)
    a = M_PI * (alpha * alpha);
    b = M_PI / (alpha * alpha);
    const double tol = (sizeof(T) >= 8 ? 2.220446049250313e-16 : 1.1920928955078125e-07) / 4;
    h = (i64)std::ceil(alpha * std::sqrt(std::log(1 / tol) / M_PI));
    w = 2 * h;
    B = (i64)std::floor(std::sqrt(std::log(1 / tol) / a) + 0.5);
    if (2 * B + 1 > 8) throw std::invalid_argument("band too wide");
    H = hvdh_halo(n, t, a, B, tol);
    K = pass ? 1 : pick_width<T>();
    G = pass ? 1 : std::max<i64>(1, cld_i(t, K * HVDH_LTARGET));
    L = cld_i(t, K * G);
    R = L + 2 * H;
    rsm = kReseed - 1;
    const double d = (double)Delta / (double)n;
    aT = (T)a;
    dT = (T)d;
    const double rcd[7] = {std::exp(2 * a), std::exp(-2 * a), std::exp(-a), std::exp(2 * a * d),
                           std::exp(-2 * a * d), std::exp(-a * (d * d)), std::exp(-2 * a * (d * d))};
    for (int k = 0; k < 7; ++k) rc[k] = (T)rcd[k];
    for (i64 dd = 1; dd <= B; ++dd) chT.push_back((T)std::exp(-a * (double)(dd * dd)));
    se.resize(G * K); sx.resize(G * K); so.resize(G * K);
    for (i64 ch = 0; ch < G * K; ++ch) {
      const i64 q0 = mod_i(ch * L - H, t);
      i64 e, l;
      hvdh_e(n, t, q0 - B, &e, &l);
      se[ch] = e;
      sx[ch] = q0;
      hvdh_e(n, t, q0, &e, &l);
      so[ch] = mod_i((i64)((__int128)Delta * l % n), n);
    }
    if (pass) tstages = build_stages<T>(t, D, false);
    else pt.reset(anyplan<T>(t, D, (T)1, 1));
    const i64 ufl = (R + B) * (B + 1) * K;
    const i64 tbytes = G * (R * B * K * (i64)sizeof(T) + ufl * (i64)sizeof(T) + R * K * 8);
    tab = pass || factors == 1 || (factors == 0 && tbytes <= HVDH_TABLE_MAX);
    if (tab) {
      lt.resize(G * K * R * B); ut.resize(G * K * R * (B + 1)); ot.resize(G * K * R);
      for (i64 ch = 0; ch < G * K; ++ch)
        factor(ch, &lt[ch * R * B], &ut[ch * R * (B + 1)], &ot[ch * R]);
    }
  }
  // column state at e, beta' = (e - n)/2n: (G, 1/G, A', Hh) = (exp(-2a beta'),
  // exp(2a beta'), exp(-a beta'^2), exp(-2a beta' delta)) (_hvdh_seed,
  // src/hvdh.jl:472-479)
  struct Col { T g, gi, A, hh; };
  Col seed(i64 e) const {
    const T beta = (T)(e - n) * (T)(1.0 / (2.0 * (double)n));
    Col s;
    s.g = vexp<T>((T)(-2) * aT * beta);
    s.gi = (T)1 / s.g;
    s.A = vexp<T>(-aT * beta * beta);
    s.hh = vexp<T>((T)(-2) * aT * dT * beta);
    return s;
  }
  // one column on: off the unknowns e -= 2n, on one e += 2 Delta
  // (_hvdh_step, src/hvdh.jl:481-496; rc = exp of 2a, -2a, -a, 2ad, -2ad, -ad^2, -2ad^2)
  void step(i64& e, Col& s) const {
    const bool hit = e < 2 * n;
    s.A *= hit ? s.hh * rc[5] : s.gi * rc[2];
    s.g *= hit ? rc[4] : rc[0];
    s.gi *= hit ? rc[3] : rc[1];
    s.hh *= hit ? rc[6] : rc[3];
    e = hit ? e + 2 * Delta : e - 2 * n;
  }
  // the band of chunk ch, built from a ring of 8 columns and eliminated row
  // by row without pivoting (_hvdh_prime!, _hvdh_row!, _hvdh_factor!:
  // src/hvdh.jl:498-560, 637-654)
  void factor(i64 ch, T* lf, T* uf, i64* ob) const {
    T rA[8], rG[8], rGi[8];  // A' (0 off the unknowns), G, 1/G per ring slot
    auto put = [&](i64 slot, i64 e, const Col& s) {
      rA[slot] = e < 2 * n ? s.A : (T)0;
      rG[slot] = s.g;
      rGi[slot] = s.gi;
    };
    i64 e = se[ch];
    Col cs = seed(e);
    for (i64 cc = -B; cc < B; ++cc) { put(cc & 7, e, cs); step(e, cs); }
    i64 on = so[ch];
    // rows -B .. -1: identity pads
    std::vector<T> U((R + B) * (B + 1), (T)0);
    for (i64 i = 0; i < B; ++i) U[i * (B + 1)] = (T)1;
    std::vector<T> r(2 * B + 1);
    for (i64 i = 0; i < R; ++i) {
      if (((i + 2 * B) & rsm) == 0) cs = seed(e);
      put((i + B) & 7, e, cs);
      step(e, cs);
      const T Aq = rA[i & 7];
      const bool hit = Aq > (T)0;
      // entry at column i + m: exp(-a m^2) A' G^m
      for (i64 m = -B; m <= B; ++m) {
        if (m == 0) { r[B] = hit ? Aq : (T)1; continue; }
        const i64 o = (i + m) & 7;
        const T gc = m > 0 ? rG[o] : rGi[o];
        T gm = gc;
        for (i64 k = 2; k <= (m < 0 ? -m : m); ++k) gm *= gc;
        r[m + B] = hit ? chT[(m < 0 ? -m : m) - 1] * rA[o] * gm : (T)0;
      }
      for (i64 k = B; k >= 1; --k) {
        const T* ur = &U[(i - k + B) * (B + 1)];
        const T fk = r[B - k] * ur[0];
        lf[i * B + (k - 1)] = fk;
        for (i64 j = 1; j <= B; ++j) r[B - k + j] = std::fma(-fk, ur[j], r[B - k + j]);
      }
      T* ur = &U[(i + B) * (B + 1)];
      ur[0] = (T)1 / r[B];
      for (i64 j = 1; j <= B; ++j) ur[j] = r[B + j];
      for (i64 j = 0; j <= B; ++j) uf[i * (B + 1) + j] = ur[j];
      ob[i] = hit ? on : -1;
      if (hit) { on += Delta; if (on >= n) on -= n; }
    }
  }
  // _hvdh_spread! (src/hvdh.jl:337-470): v[q] = sum over taps o of
  // exp(-b (delta_q - o)^2) / alpha * ys[(q + (o - 1) Delta) mod n],
  // delta_q = (t - q) / t, o = 1 - w/2 .. w/2, rows q = i Delta + j in blocks
  // of J rows, V lanes along j; per lane E = exp(-b delta^2)/alpha, G =
  // exp(2b delta), 1/G, R = exp(2b kappa delta - b kappa^2), Hr = exp(2b
  // theta delta) advance by constant factors per vector and are re-seeded
  // every kSReseed vectors; row g's weights follow row 0's by Hr and
  // constants; tap weights E G^o exp(-b o^2), the centre tap first, then
  // o = 1, 2, .., then o = -1, -2, ...
  void spread_rec(const std::vector<T>& ys, std::vector<T>& v) const {
    const i64 V = pick_width<T>(), J = kJ, rs = kSReseed, hw = w / 2;
    const double th = (double)Delta / (double)t, ka = (double)V / (double)t;
    const T fE = (T)std::exp(-2 * b * (ka * ka)), fG = (T)std::exp(-2 * b * ka), fGi = (T)std::exp(2 * b * ka),
            fH = (T)std::exp(-2 * b * th * ka);
    std::vector<T> kc(w + 1);  // kc[o + hw], o = 1 - hw .. hw
    for (i64 o = 1 - hw; o <= hw; ++o) kc[o + hw] = (T)std::exp(-b * (double)(o * o));
    std::vector<T> gc1(J), gc2(J), gc3(J);
    for (i64 g = 0; g < J; ++g) {
      const double gt = (double)g * th;
      gc1[g] = (T)std::exp(-b * (gt * gt));
      gc2[g] = (T)std::exp(-2 * b * (double)g * th);
      gc3[g] = (T)std::exp(2 * b * (double)g * th);
    }
    const T bT = (T)b, b2T = (T)(2 * b), rkT = (T)(2 * b * ka), rk2T = (T)(b * (ka * ka)), hT = (T)(2 * b * th);
    const T it = (T)(1.0 / (double)t), ia = (T)(1.0 / alpha);
    const i64 nseg = cld_i(Delta, rs * V);
    const i64 nblk = cld_i(cld_i(t, Delta), J);
    std::vector<T> E(V), Gv(V), Gi(V), Rv(V), Hv(V);
    for (i64 ib = 0; ib < nblk; ++ib)
      for (i64 seg = 0; seg < nseg; ++seg) {
        const i64 i0 = J * ib;
        i64 j = seg * rs * V;
        const i64 jend = std::min(Delta, j + rs * V);
        for (i64 blk = 0; j < jend; j += V, ++blk) {
          if ((blk & (rs - 1)) == 0)
            for (i64 s = 0; s < V; ++s) {
              const T dl = (T)((t - i0 * Delta - j) - s) * it;
              E[s] = vexp<T>(-bT * dl * dl) * ia;
              Gv[s] = vexp<T>(b2T * dl);
              Gi[s] = vexp<T>(-b2T * dl);
              Rv[s] = vexp<T>(rkT * dl - rk2T);
              Hv[s] = vexp<T>(hT * dl);
            }
          for (i64 s = 0; s < V; ++s) {
            T F = E[s];
            for (i64 g = 0; g < J; ++g) {
              if (g > 0) F *= Hv[s];
              const i64 lim = std::min(std::max<i64>(t - (i0 + g) * Delta, 0), Delta);
              if (j + s >= lim) continue;  // past the row's end or t
              const T Eg = F * gc1[g], Gg = Gv[s] * gc2[g], Gig = Gi[s] * gc3[g];
              auto at = [&](i64 o) { return mod_i((i0 + g + o - 1) * Delta + j + s, n); };
              const i64 m0 = at(0);
              T re = Eg * ys[2 * m0], im = Eg * ys[2 * m0 + 1];
              T P = Eg;
              for (i64 o = 1; o <= hw; ++o) {
                P *= Gg;
                const T W = P * kc[o + hw];
                const i64 m = at(o);
                re = std::fma(W, ys[2 * m], re);
                im = std::fma(W, ys[2 * m + 1], im);
              }
              P = Eg;
              for (i64 o = -1; o >= 1 - hw; --o) {
                P *= Gig;
                const T W = P * kc[o + hw];
                const i64 m = at(o);
                re = std::fma(W, ys[2 * m], re);
                im = std::fma(W, ys[2 * m + 1], im);
              }
              const i64 q = (i0 + g) * Delta + j + s;
              v[2 * q] = re; v[2 * q + 1] = im;
            }
          }
          for (i64 s = 0; s < V; ++s) {
            E[s] *= Rv[s];
            Rv[s] *= fE;
            Gv[s] *= fG;
            Gi[s] *= fGi;
            Hv[s] *= fH;
          }
        }
      }
  }
  // HvPass's tabulated weights T(exp(-b (delta_q - o)^2) / alpha), summed
  // tap by tap from o = 1 - w/2 (_hv_parts, _rows_spread!: src/hvdh.jl:
  // 743-750, 856-871)
  void spread_tab(const std::vector<T>& ys, std::vector<T>& v) const {
    const i64 hw = w / 2;
    for (i64 q = 0; q < t; ++q) {
      const double dq = (double)(t - q) / (double)t;
      T re = 0, im = 0;
      for (i64 o = 1 - hw; o <= hw; ++o) {
        const double d = dq - (double)o;
        const T wt = (T)(std::exp(-b * (d * d)) / alpha);
        const i64 m = mod_i(q + (o - 1) * Delta, n);
        re = std::fma(wt, ys[2 * m], re);
        im = std::fma(wt, ys[2 * m + 1], im);
      }
      v[2 * q] = re; v[2 * q + 1] = im;
    }
  }
  void exec(const void* xv, void* yv) override {
    const T* x = (const T*)xv;
    T* y = (T*)yv;
    // _hvdh_scatter! (src/hvdh.jl:246-294): ys[l Delta mod n] = u_l
    std::vector<T> ys(2 * n);
    for (i64 l = 0; l < n; ++l) {
      const i64 m = (i64)((__int128)l * Delta % n);
      ys[2 * m] = x[2 * l]; ys[2 * m + 1] = x[2 * l + 1];
    }
    std::vector<T> v(2 * t), Y(2 * t);
    if (pass_form) {
      spread_tab(ys, v);
      std::vector<T> are(t), aim(t), bre(t), bim(t);
      for (i64 q = 0; q < t; ++q) { are[q] = v[2 * q]; aim[q] = v[2 * q + 1]; }
      const bool sw = run_chain(are.data(), aim.data(), bre.data(), bim.data(), tstages, 0, tstages.size(), t, 1, 1,
                                D, 1);
      const T* cr = sw ? bre.data() : are.data();
      const T* ci = sw ? bim.data() : aim.data();
      for (i64 q = 0; q < t; ++q) { Y[2 * q] = cr[q]; Y[2 * q + 1] = ci[q]; }
    } else {
      spread_rec(ys, v);
      pt->exec(v.data(), Y.data());
    }
    // _hvdh_groups! -> _hvdh_subst! / _hvdh_group!, _hvdh_back!
    // (src/hvdh.jl:232-240, 560-686)
    std::vector<T> lf, uf;
    std::vector<i64> ob;
    if (!tab) { lf.resize(R * B); uf.resize(R * (B + 1)); ob.resize(R); }
    std::vector<T> zr(R + 2 * B), zi(R + 2 * B);
    const T sc = pass_form ? (T)((double)n / (double)t) : scale * (T)n / (T)t;
    for (i64 ch = 0; ch < G * K; ++ch) {
      const T* L_ = tab ? &lt[ch * R * B] : lf.data();
      const T* U_ = tab ? &ut[ch * R * (B + 1)] : uf.data();
      const i64* O_ = tab ? &ot[ch * R] : ob.data();
      if (!tab) factor(ch, lf.data(), uf.data(), ob.data());
      std::fill(zr.begin(), zr.end(), (T)0);
      std::fill(zi.begin(), zi.end(), (T)0);
      i64 idx = sx[ch];
      for (i64 i = 0; i < R; ++i) {
        T ar = 0, ai = 0;
        if (O_[i] >= 0) { ar = Y[2 * idx]; ai = Y[2 * idx + 1]; }
        for (i64 k = B; k >= 1; --k) {
          const T f = L_[i * B + (k - 1)];
          ar = std::fma(-f, zr[i - k + B], ar);
          ai = std::fma(-f, zi[i - k + B], ai);
        }
        zr[i + B] = ar; zi[i + B] = ai;
        if (++idx >= t) idx -= t;
      }
      for (i64 i = R - 1; i >= H; --i) {
        const T* ur = U_ + i * (B + 1);
        T xr = zr[i + B], xi = zi[i + B];
        for (i64 j = 1; j <= B; ++j) {
          xr = std::fma(-ur[j], zr[i + B + j], xr);
          xi = std::fma(-ur[j], zi[i + B + j], xi);
        }
        xr *= ur[0]; xi *= ur[0];
        zr[i + B] = xr; zi[i + B] = xi;
        if (i < H + L && O_[i] >= 0) { y[2 * O_[i]] = xr * sc; y[2 * O_[i] + 1] = xi * sc; }
      }
    }
  }
  void info(std::vector<i64>& vv) override {
    vv.push_back(route); vv.push_back(n); vv.push_back(t); vv.push_back(w); vv.push_back(B); vv.push_back(H);
    vv.push_back(L); vv.push_back(G * K); vv.push_back(tab ? 1 : 2);
  }
};

// smooth part s (2, 3, 5, 7) of n (_smooth_part, src/composite.jl:43-51)
static i64 smooth_part(i64 n) {
  i64 s = 1;
  for (int f : {2, 3, 5, 7})
    while (n % (s * f) == 0) s *= f;
  return s;
}
static const i64 COMPOSITE_MIN_S = 16;    // src/composite.jl:37
static const i64 COMPOSITE_HV_MINP = 500;  // src/composite.jl:42
template <typename T>
static bool use_composite(i64 n) {  // src/composite.jl:53-54
  return n >= (sizeof(T) >= 8 ? 4096 : 32768) && smooth_part(n) >= COMPOSITE_MIN_S;
}
template <typename T>
static bool use_split(i64 n) {  // src/composite.jl:131-135
  const i64 s = smooth_part(n);
  return n % 2 == 0 && s < COMPOSITE_MIN_S && use_hvdh<T>(n / s) && n >= (sizeof(T) >= 8 ? 16384 : 65536);
}

// w_n^e (sign D) as the reference's two-level product hi[e / K] lo[e % K]
// (_tw2, src/composite.jl:275-279; tables src/composite.jl:61-73)
template <typename T>
struct TwoLevel {
  i64 n, K;
  std::vector<T> hir, hii, lor, loi;
  TwoLevel(i64 n_, int D) : n(n_) {
    K = isqrt_(n - 1) + 1;
    const i64 nh = (n + K - 1) / K;
    hir.resize(nh); hii.resize(nh); lor.resize(K); loi.resize(K);
    for (i64 i = 0; i < nh; ++i) {
      double s, co;
      sincospi((double)(2 * D * i * K) / (double)n, &s, &co);
      hir[i] = (T)co; hii[i] = (T)s;
    }
    for (i64 i = 0; i < K; ++i) {
      double s, co;
      sincospi((double)(2 * D * i) / (double)n, &s, &co);
      lor[i] = (T)co; loi[i] = (T)s;
    }
  }
  void at(i64 e, T* wr, T* wi) const {
    const i64 hi = e / K, lo = e % K;
    *wr = hir[hi] * lor[lo] - hii[hi] * loi[lo];
    *wi = hir[hi] * loi[lo] + hii[hi] * lor[lo];
  }
};

// Lane twiddles lv[W r + l] = w_n^(r l), l < W lanes (src/composite.jl:
// 76-80, 162-167).
template <typename T>
struct LaneTw {
  i64 W;
  std::vector<T> lr, li;
  LaneTw(i64 n, i64 rows, int D) : W(pick_width<T>()) {
    lr.resize(W * rows); li.resize(W * rows);
    for (i64 r = 0; r < rows; ++r)
      for (i64 l = 0; l < W; ++l) {
        double sn, cs;
        sincospi((double)(2 * D * (r * l)) / (double)n, &sn, &cs);
        lr[W * r + l] = (T)cs; li[W * r + l] = (T)sn;
      }
  }
};

// x (c w_n^(r k)) for lane k of a run of L lanes from lane0, as FFTJ's
// W-lane windows build it (_rows_scale_tw!, _split_twiddle!:
// src/composite.jl:239-301): the window's first lane k0 by the two-level
// table, times the lane twiddle w_n^(r (k - k0)), with c folded in; windows
// step by W and the last one overlaps the previous, its values the ones
// kept. Runs shorter than W take the scalar form c (x w).
template <typename T>
static void tw_window(const TwoLevel<T>& tw, const LaneTw<T>& lv, T c, i64 r, i64 k, i64 lane0, i64 L, T xr, T xi,
                      T* yr, T* yi) {
  const i64 W = lv.W;
  if (W > 1 && L >= W) {
    const i64 rel = k - lane0;
    const i64 k0 = lane0 + (rel >= L - W ? L - W : rel / W * W);
    T ar, ai;
    tw.at(r * k0, &ar, &ai);
    const T vr = lv.lr[W * r + (k - k0)], vi = lv.li[W * r + (k - k0)];
    const T car = c * ar, cai = c * ai;
    const T twr = std::fma(car, vr, -(cai * vi));
    const T twi = std::fma(car, vi, cai * vr);
    *yr = std::fma(xr, twr, -(xi * twi));
    *yi = std::fma(xr, twi, xi * twr);
  } else {
    T wr, wi;
    tw.at(r * k, &wr, &wi);
    *yr = c * (xr * wr - xi * wi);
    *yi = c * (xr * wi + xi * wr);
  }
}

// lanes per chunk of a batched resampling pass over B lanes whose work
// rows number M (_rs_pass / _hv_pass, src/resample.jl:453-461,
// src/hvdh.jl:752-755); the last chunk takes the rest
static const i64 RS_CHUNK_MAX = 1 << 19;
template <typename T>
static i64 rs_chunk_lanes(i64 M, i64 B) {
  const i64 W = pick_width<T>();
  if (B < 2 * W) return B;
  const i64 c = RS_CHUNK_MAX / (4 * M * (i64)sizeof(T)) / W * W;
  return std::min(std::max(c, W), B / W * W);
}

// CompositePlan (src/composite.jl:10-101): n = p s, j = j1 + p j2,
// k = k2 + s k1: length-s transforms over j2 (batch p), twiddles
// w_n^(j1 k2), then the length-p transforms over j1 for each k2 by
// resampling -- batched HvdH (HvPass) for p >= 500, else batched
// oversampled resampling (RsPass). The restatement runs each lane's
// length-p transform through HvdhPlan's pass form, the HvPass arithmetic
// for one lane (tabulated weights, one cyclic band, the no-small chain).
template <typename T>
struct CompositePlan : PlanBase {
  int D;
  T scale;
  i64 p, s;
  std::vector<Stage<T>> stages;
  std::unique_ptr<HvdhPlan<T>> hv;
  std::unique_ptr<RsPass<T>> rs;
  TwoLevel<T> tw;
  std::unique_ptr<LaneTw<T>> lv;
  CompositePlan(i64 n_, int D_, T scale_) : D(D_), scale(scale_), tw(n_, D_) {
    n = n_;
    route = ORC_COMPOSITE;
    s = smooth_part(n);
    p = n / s;
    lv.reset(new LaneTw<T>(n, p, D));
    stages = build_stages<T>(s, D, false);
    if (p >= COMPOSITE_HV_MINP) hv.reset(new HvdhPlan<T>(p, D, (T)1, 1, true));
    else rs.reset(new RsPass<T>(p, D, s));
  }
  void exec(const void* xv, void* yv) override {
    const T* x = (const T*)xv;
    T* y = (T*)yv;
    std::vector<T> are(n), aim(n), bre(n), bim(n);
    for (i64 i = 0; i < n; ++i) { are[i] = x[2 * i]; aim[i] = x[2 * i + 1]; }
    const bool sw = run_chain(are.data(), aim.data(), bre.data(), bim.data(), stages, 0, stages.size(), s, 1, p, D, 1);
    const T* cre = sw ? bre.data() : are.data();
    const T* cim = sw ? bim.data() : aim.data();
    // c[j1 + p k2] -> o[k2 + s j1]; the twiddle w_n^(j1 k2) is applied in
    // the resampling pass's load, per chunk of lanes (_rs_chunk! /
    // _hv_chunk! with _rows_scale_tw!)
    std::vector<T> ore(n), oim(n);
    for (i64 k2 = 0; k2 < s; ++k2)
      for (i64 j1 = 0; j1 < p; ++j1) { ore[k2 + s * j1] = cre[j1 + p * k2]; oim[k2 + s * j1] = cim[j1 + p * k2]; }
    const i64 M = rs ? rs->m : std::max(hv->t, hv->R + 2 * hv->B);
    const i64 C = rs_chunk_lanes<T>(M, s), nc = std::max<i64>(1, s / C);
    auto chunk = [&](i64 k2, i64* lane0, i64* L) {
      const i64 c = std::min(k2 / C, nc - 1);
      *lane0 = c * C;
      *L = c == nc - 1 ? s - c * C : C;
    };
    if (rs) {
      rs->run(ore.data(), oim.data(), 0, D, [&](i64 j1, i64 k2, T c, T xr, T xi, T* yr, T* yi) {
        i64 lane0, L;
        chunk(k2, &lane0, &L);
        tw_window(tw, *lv, c, j1, k2, lane0, L, xr, xi, yr, yi);
      });  // rows j1 of s lanes k2, in place: rows k1
      for (i64 i = 0; i < n; ++i) { y[2 * i] = ore[i] * scale; y[2 * i + 1] = oim[i] * scale; }
    } else {
      std::vector<T> lin(2 * p), lout(2 * p);
      for (i64 k2 = 0; k2 < s; ++k2) {
        i64 lane0, L;
        chunk(k2, &lane0, &L);
        for (i64 j1 = 0; j1 < p; ++j1)
          tw_window(tw, *lv, (T)1, j1, k2, lane0, L, ore[k2 + s * j1], oim[k2 + s * j1], &lin[2 * j1], &lin[2 * j1 + 1]);
        hv->exec(lin.data(), lout.data());
        for (i64 k1 = 0; k1 < p; ++k1) {
          y[2 * (k2 + s * k1)] = lout[2 * k1] * scale;
          y[2 * (k2 + s * k1) + 1] = lout[2 * k1 + 1] * scale;
        }
      }
    }
  }
  void info(std::vector<i64>& v) override { v.push_back(route); v.push_back(n); v.push_back(p); v.push_back(s); }
};

// SplitPlan (src/composite.jl:103-280): decimation in time, x_r[j] =
// x[r + s j]; s length-p HvdH transforms (unnormalized); planes
// p r + k1 <- w_n^(r k1) Y_r[k1]; the length-s chain over r (batch p)
// writes X[k1 + p k2] in natural order.
template <typename T>
struct SplitPlan : PlanBase {
  int D;
  T scale;
  i64 p, s;
  std::unique_ptr<HvdhPlan<T>> hv;
  std::vector<Stage<T>> stages;
  TwoLevel<T> tw;
  std::unique_ptr<LaneTw<T>> lv;
  SplitPlan(i64 n_, int D_, T scale_) : D(D_), scale(scale_), tw(n_, D_) {
    n = n_;
    route = ORC_SPLIT;
    s = smooth_part(n);
    p = n / s;
    lv.reset(new LaneTw<T>(n, s, D));
    hv.reset(new HvdhPlan<T>(p, D, (T)1, 0));
    stages = build_stages<T>(s, D, false);
  }
  void exec(const void* xv, void* yv) override {
    const T* x = (const T*)xv;
    T* y = (T*)yv;
    std::vector<T> xs(2 * p), ys(2 * p), are(n), aim(n), bre(n), bim(n);
    for (i64 r = 0; r < s; ++r) {
      for (i64 j = 0; j < p; ++j) { xs[2 * j] = x[2 * (s * j + r)]; xs[2 * j + 1] = x[2 * (s * j + r) + 1]; }
      hv->exec(xs.data(), ys.data());
      for (i64 k1 = 0; k1 < p; ++k1)  // _split_twiddle! (src/composite.jl:237-266)
        tw_window(tw, *lv, (T)1, r, k1, 0, p, ys[2 * k1], ys[2 * k1 + 1], &are[p * r + k1], &aim[p * r + k1]);
    }
    const bool sw = run_chain(are.data(), aim.data(), bre.data(), bim.data(), stages, 0, stages.size(), s, 1, p, D, 1);
    const T* cre = sw ? bre.data() : are.data();
    const T* cim = sw ? bim.data() : aim.data();
    for (i64 i = 0; i < n; ++i) { y[2 * i] = cre[i] * scale; y[2 * i + 1] = cim[i] * scale; }
  }
  void info(std::vector<i64>& v) override { v.push_back(route); v.push_back(n); v.push_back(p); v.push_back(s); }
};

// _anyplan routing (src/plan.jl:192-206)
template <typename T>
static PlanBase* anyplan(i64 n, int D, T scale, int nthreads) {
  if (n < 1) throw std::runtime_error("transform length must be positive");
  if (!factor_radices(n).ok) {
    if (use_composite<T>(n)) return new CompositePlan<T>(n, D, scale);
    if (use_hvdh<T>(n)) return new HvdhPlan<T>(n, D, scale, 0);
    if (use_split<T>(n)) return new SplitPlan<T>(n, D, scale);
    return new ResamplePlan<T>(n, D, scale);
  }
  if (use_ragged<T>(n, nthreads > 1)) return new FourStepPlan<T>(n, D, scale, nthreads);
  if (slow_smooth<T>(n)) return new ResamplePlan<T>(n, D, scale);
  if (use_fourstep<T>(n, nthreads > 1 && n >= 2 * FS_TASK_MIN)) return new FourStepPlan<T>(n, D, scale, nthreads);
  return new FFTPlan<T>(n, D, scale, nthreads);
}

template <typename T>
struct DimPass {
  i64 nd, Bi, Bo;
  std::vector<Stage<T>> stages;
  std::unique_ptr<RsPass<T>> fb;
};

// _use_fs2 (src/fourstep.jl:518-529): a 2-D n1 x n2 transform runs as
// Fs2Plan -- the strided dim 2 in strips first, then each contiguous row
// ending in a fused power-of-two stage -- from 1 MB threaded / 4 MB serial.
static const i64 FS2_MIN_BYTES = 1 << 20;  // _FS2_MIN_BYTES
template <typename T>
static bool use_fs2(i64 n1, i64 n2, bool threaded) {
  const i64 bytes = 2 * n1 * n2 * (i64)sizeof(T);
  if (bytes < (threaded ? FS2_MIN_BYTES : 4 * FS2_MIN_BYTES)) return false;
  const int W = pick_width<T>();
  if (!threaded && n1 % ((i64)fs_width<T>(n2) * W) != 0) return false;
  if (4 * (i64)W * n2 * (i64)sizeof(T) > FS_INNER_MAX) return false;
  i64 N1 = 0, N2 = 0;
  if (!fourstep_split<T>(n1 * n2, 1, n2, &N1, &N2)) return false;
  if (!factor_radices(n1).ok || !factor_radices(n2).ok) return false;
  const std::vector<Stage<T>> rows = build_stages<T>(n1, -1, true);
  const int f = rows.back().radix;
  return (f == 2 || f == 4 || f == 8) && n1 / f >= W;
}

// pencil_fused (src/ndplan.jl:46-54): would a per-pencil chain of length n,
// built with the small-stride layout allowed, get the fused-edge 1-D
// treatment? Its first stage is small when use_small (src/plan.jl:9-11)
// holds at stride 1: radix 4 with n/4 a whole number of vectors.
template <typename T>
static bool pencil_fused(i64 n, const std::vector<Stage<T>>& stages) {
  const int W = pick_width<T>();
  if (stages.empty()) return false;
  const int f = stages.back().radix;
  const i64 slast = (f == 2 || f == 4 || f == 8) ? n / f : 0;
  const bool small0 = stages[0].radix == 4 && 1 < W && n / 4 >= W && (n / 4) % W == 0;
  return W > 1 && stages.size() >= 2 && stages[0].radix == 4 && small0 && (n >> 2) % W == 0 && slast >= W &&
         slast % W == 0;
}

// _real_batched (src/ndplan.jl:343-353): the N-d real edge along dim 1 runs
// batched (pencils as lanes, half-length chain without the small-stride
// layout) when the half length is smooth and the batch fills the vector
// lanes, unless the per-pencil chain is fused -- then only for 16-lane
// vectors with an L2-resident working set.
template <typename T>
static bool real_batched(i64 n1, i64 B) {
  const int W = pick_width<T>();
  if (!(W > 1 && n1 % 2 == 0 && n1 >= 2 && B >= W)) return false;
  const i64 h = n1 >> 1;
  if (!factor_radices(h).ok) return false;
  if (!pencil_fused<T>(h, build_stages<T>(h, -1, true))) return true;
  return W >= 16 && (h + 1) * B * (i64)sizeof(T) <= ((i64)1 << 19);
}

template <typename T>
struct NdPlan : PlanBase {
  int D;
  T scale;
  std::vector<i64> dims;
  i64 len;
  int nt;
  bool fs2 = false;  // 2-D plan in Fs2Plan order (use_fs2)
  bool dim1_batched = false;  // the dim-1 pass runs the no-small chain with pencils as lanes
  std::vector<std::unique_ptr<DimPass<T>>> passes;
  std::vector<T> are, aim, bre, bim;
  // _ndplan (src/ndplan.jl:57-118); dims before first_dim are pure batch
  NdPlan(const std::vector<i64>& dims_, int D_, T scale_, int nthreads, int first_dim = 0)
      : D(D_), scale(scale_), dims(dims_) {
    route = -1;
    len = 1;
    for (i64 d : dims) { if (d < 1) throw std::runtime_error("dimensions must be positive"); len *= d; }
    n = len;
    nt = plan_tasks(len, nthreads);
    int W = pick_width<T>();
    for (size_t d = first_dim; d < dims.size(); ++d) {
      i64 nd = dims[d];
      if (nd == 1) continue;
      i64 Bi = 1, Bo = 1;
      for (size_t e = 0; e < d; ++e) Bi *= dims[e];
      for (size_t e = d + 1; e < dims.size(); ++e) Bo *= dims[e];
      std::unique_ptr<DimPass<T>> ps(new DimPass<T>());
      ps->nd = nd; ps->Bi = Bi; ps->Bo = Bo;
      if (factor_radices(nd).ok) {
        ps->stages = build_stages<T>(nd, D, Bi == 1);
        // a dim-1 chain without the fused edge runs transposed, pencils as
        // lanes, on the chain built without the small-stride layout
        // (src/ndplan.jl:72-77); the transposes move data only, so each
        // pencil here runs that chain in place of the transposed sweep
        if (Bi == 1 && Bo >= W && !pencil_fused<T>(nd, ps->stages)) {
          ps->stages = build_stages<T>(nd, D, false);
          if (passes.empty()) dim1_batched = true;
        }
      } else {
        ps->fb.reset(new RsPass<T>(nd, D, Bi == 1 ? Bo : Bi));
      }
      passes.push_back(std::move(ps));
    }
    route = ORC_NDPLAN;
    // N == 2 from dim 1 (_ndplan, src/ndplan.jl:112-113): FFTJ's NdPlan then
    // executes through its Fs2Plan -- the same two chains, dim 2 first
    if (dims.size() == 2 && first_dim == 0 && passes.size() == 2 && !passes[0]->fb && !passes[1]->fb &&
        use_fs2<T>(dims[0], dims[1], nt > 1)) {
      fs2 = true;
      route = ORC_FS2;
      // Fs2Plan's rows are the length-n1 chain as a 1-D plan builds it
      // (src/fourstep.jl:531-536)
      passes[0]->stages = build_stages<T>(dims[0], D, true);
      dim1_batched = false;
      std::swap(passes[0], passes[1]);
    }
    are.resize(len); aim.resize(len); bre.resize(len); bim.resize(len);
  }
  // split planes in (cre, cim); returns the plane pair holding the result
  void core(T*& cre, T*& cim, T*& ore, T*& oim) {
    for (auto& pp : passes) {
      DimPass<T>& ps = *pp;
      if (ps.fb) {
        if (ps.Bi == 1 && ps.Bo > 1) {
          // dim 1: transpose so pencils become lanes (src/ndplan.jl:137-151)
          for (i64 o = 0; o < ps.Bo; ++o)
            for (i64 j = 0; j < ps.nd; ++j) { ore[ps.Bo * j + o] = cre[ps.nd * o + j]; oim[ps.Bo * j + o] = cim[ps.nd * o + j]; }
          ps.fb->run(ore, oim, 0, D);
          for (i64 o = 0; o < ps.Bo; ++o)
            for (i64 j = 0; j < ps.nd; ++j) { cre[ps.nd * o + j] = ore[ps.Bo * j + o]; cim[ps.nd * o + j] = oim[ps.Bo * j + o]; }
        } else {
          for (i64 o = 0; o < ps.Bo; ++o) ps.fb->run(cre, cim, o * ps.Bi * ps.nd, D);
        }
        continue;
      }
      i64 block = ps.Bi * ps.nd;
      bool sw = false;
      for (i64 o = 0; o < ps.Bo; ++o)
        sw = run_chain(cre + o * block, cim + o * block, ore + o * block, oim + o * block, ps.stages, 0,
                       ps.stages.size(), ps.nd, 1, ps.Bi, D, nt);
      if (sw) { std::swap(cre, ore); std::swap(cim, oim); }
    }
  }
  void exec(const void* xv, void* yv) override {
    const T* x = (const T*)xv;
    T* y = (T*)yv;
    T *cre = are.data(), *cim = aim.data(), *ore = bre.data(), *oim = bim.data();
    for (i64 c = 0; c < len; ++c) { cre[c] = x[2 * c]; cim[c] = x[2 * c + 1]; }
    core(cre, cim, ore, oim);
    for (i64 c = 0; c < len; ++c) { y[2 * c] = cre[c] * scale; y[2 * c + 1] = cim[c] * scale; }
  }
};

// RfftNdPlan / IrfftNdPlan (src/ndplan.jl:355-519). The real edge along
// dim 1 runs per pencil through the 1-D real plan, or -- when real_batched
// holds -- batched: the half-length chain built without the small-stride
// layout on every pencil, then the split/merge post-pass (pre-pass for the
// inverse) with the 1-D plan's twiddles. FFTJ runs the batched form on
// transposed planes with the pencils as vector lanes; the transposes move
// data only, so each pencil here runs the same arithmetic in its own row.
template <typename T>
struct RfftNd {
  std::vector<i64> rdims, cdims;
  i64 B;
  bool batched;
  std::vector<Stage<T>> bstages;  // forward chain for h = n1/2 (no small layout)
  std::unique_ptr<RfftPlan<T>> r1;  // 1-D plan (twiddle source when batched)
  std::unique_ptr<NdPlan<T>> rest;
  std::vector<T> C, are, aim, bre, bim;
  RfftNd(const std::vector<i64>& dims, int nthreads) : rdims(dims) {
    cdims = dims;
    cdims[0] = dims[0] / 2 + 1;
    B = 1;
    for (size_t d = 1; d < dims.size(); ++d) B *= dims[d];
    batched = real_batched<T>(dims[0], B);
    r1.reset(new RfftPlan<T>(dims[0], nthreads));
    rest.reset(new NdPlan<T>(cdims, -1, (T)1, nthreads, 1));
    C.resize(2 * cdims[0] * B);
    if (batched) {
      const i64 h = dims[0] / 2;
      bstages = build_stages<T>(h, -1, false);
      are.resize(h); aim.resize(h); bre.resize(h); bim.resize(h);
    }
  }
  void exec(const T* X, T* Y) {
    i64 n1 = rdims[0], h1p = cdims[0];
    if (!batched) {
      for (i64 o = 0; o < B; ++o) r1->exec(X + o * n1, C.data() + 2 * o * h1p);
    } else {
      const i64 h = n1 / 2;
      const T half = (T)0.5;
      for (i64 o = 0; o < B; ++o) {
        const T* x = X + o * n1;
        for (i64 j = 0; j < h; ++j) { are[j] = x[2 * j]; aim[j] = x[2 * j + 1]; }
        bool sw = run_chain(are.data(), aim.data(), bre.data(), bim.data(), bstages, 0, bstages.size(), h, 1, 1,
                            -1, 1);
        const T* zr = sw ? bre.data() : are.data();
        const T* zi = sw ? bim.data() : aim.data();
        T* y = C.data() + 2 * o * h1p;
        // _rfft_post_range! (src/stockham.jl:590-614)
        y[0] = zr[0] + zi[0]; y[1] = 0;
        y[2 * h] = zr[0] - zi[0]; y[2 * h + 1] = 0;
        for (i64 k = 1; k < h; ++k) {
          T ar = zr[k], ai = zi[k];
          T br = zr[h - k], bi = -zi[h - k];
          T xer = (ar + br) * half, xei = (ai + bi) * half;
          T xor_ = (ar - br) * half, xoi = (ai - bi) * half;
          T wr = r1->twr[k], wi = r1->twi[k];
          y[2 * k] = xer + std::fma(wr, xoi, wi * xor_);
          y[2 * k + 1] = xei + std::fma(wi, xoi, -(wr * xor_));
        }
      }
    }
    rest->exec(C.data(), Y);
  }
};
template <typename T>
struct IrfftNd {
  std::vector<i64> rdims, cdims;
  i64 B;
  bool batched;
  T bpre = (T)1;                  // batched pre-pass factor, every normalization folded in
  std::vector<Stage<T>> bstages;  // backward chain for h = n1/2 (no small layout)
  std::unique_ptr<IrfftPlan<T>> r1;
  std::unique_ptr<NdPlan<T>> rest;
  std::vector<T> C, are, aim, bre, bim;
  IrfftNd(const std::vector<i64>& dims, bool normalized, int nthreads) : rdims(dims) {
    cdims = dims;
    cdims[0] = dims[0] / 2 + 1;
    B = 1;
    for (size_t d = 1; d < dims.size(); ++d) B *= dims[d];
    T restscale = normalized ? (T)1 / (T)B : (T)1;
    batched = real_batched<T>(dims[0], B);
    r1.reset(new IrfftPlan<T>(dims[0], normalized, nthreads));
    // the batched form skips the rest chain's output scale and the 1-D
    // plan's normalization: 1/(n1 B) = restscale / n1 goes into the pre-pass
    // (src/ndplan.jl:466-469)
    if (batched) {
      bpre = normalized ? restscale / (T)dims[0] : (T)1;
      restscale = (T)1;
      const i64 h = dims[0] / 2;
      bstages = build_stages<T>(h, +1, false);
      are.resize(h); aim.resize(h); bre.resize(h); bim.resize(h);
    }
    rest.reset(new NdPlan<T>(cdims, +1, restscale, nthreads, 1));
    C.resize(2 * cdims[0] * B);
  }
  void exec(const T* X, T* y) {
    i64 n1 = rdims[0], h1p = cdims[0];
    rest->exec(X, C.data());
    if (!batched) {
      for (i64 o = 0; o < B; ++o) r1->exec(C.data() + 2 * o * h1p, y + o * n1);
      return;
    }
    const i64 h = n1 / 2;
    const T pv = bpre;
    for (i64 o = 0; o < B; ++o) {
      const T* x = C.data() + 2 * o * h1p;
      // _irfft_pre_range! (src/stockham.jl:633-655)
      for (i64 k = 0; k < h; ++k) {
        T ar = x[2 * k], ai = x[2 * k + 1];
        T br = x[2 * (h - k)], bi = -x[2 * (h - k) + 1];
        T xer = (ar + br) * pv, xei = (ai + bi) * pv;
        T xdr = (ar - br) * pv, xdi = (ai - bi) * pv;
        T wr = r1->twr[k], wi = r1->twi[k];
        T tr = std::fma(wr, xdr, -(wi * xdi));
        T ti = std::fma(wr, xdi, wi * xdr);
        are[k] = xer - ti;
        aim[k] = xei + tr;
      }
      bool sw = run_chain(are.data(), aim.data(), bre.data(), bim.data(), bstages, 0, bstages.size(), h, 1, 1, +1,
                          1);
      const T* zr = sw ? bre.data() : are.data();
      const T* zi = sw ? bim.data() : aim.data();
      T* yo = y + o * n1;
      for (i64 j = 0; j < h; ++j) { yo[2 * j] = zr[j]; yo[2 * j + 1] = zi[j]; }
    }
  }
};

// ---- FP64 direct DFT with double-double accumulation -----------------------
static inline void two_sum(double a, double b, double* s, double* e) {
  *s = a + b;
  double bb = *s - a;
  *e = (a - (*s - bb)) + (b - bb);
}
static void dft_f64(i64 n, const double* x, double* y, int sign) {
  std::vector<double> cr(n), ci(n);
  for (i64 k = 0; k < n; ++k) {
    double s, c;
    sincospi((double)(2 * k) / (double)n, &s, &c);
    cr[k] = c; ci[k] = sign * s;
  }
  for (i64 k = 0; k < n; ++k) {
    double sr = 0, er = 0, si = 0, ei = 0;
    for (i64 j = 0; j < n; ++j) {
      i64 e = (i64)(((__int128)j * k) % n);
      double wr = cr[e], wi = ci[e];
      double xr = x[2 * j], xi = x[2 * j + 1];
      // products with their rounding errors (fma), then compensated sums
      double p1 = wr * xr, p1e = std::fma(wr, xr, -p1);
      double p2 = -(wi * xi), p2e = -std::fma(wi, xi, -(wi * xi));
      double p3 = wr * xi, p3e = std::fma(wr, xi, -p3);
      double p4 = wi * xr, p4e = std::fma(wi, xr, -p4);
      double t, te;
      two_sum(sr, p1, &t, &te); sr = t; er += te + p1e;
      two_sum(sr, p2, &t, &te); sr = t; er += te + p2e;
      two_sum(si, p3, &t, &te); si = t; ei += te + p3e;
      two_sum(si, p4, &t, &te); si = t; ei += te + p4e;
    }
    y[2 * k] = sr + er;
    y[2 * k + 1] = si + ei;
  }
}

}  // namespace orc

using namespace orc;

// ---------------------------------------------------------------------------
// C ABI of the oracle.
namespace {
struct Handle {
  int dtype = 0;
  int kind = 0;  // 0 c2c, 1 rfft, 2 irfft, 3 nd, 4 rfft nd, 5 irfft nd
  std::unique_ptr<PlanBase> p32, p64;
  std::unique_ptr<RfftPlan<float>> r32;
  std::unique_ptr<RfftPlan<double>> r64;
  std::unique_ptr<IrfftPlan<float>> i32;
  std::unique_ptr<IrfftPlan<double>> i64_;
  std::unique_ptr<RfftNd<float>> rn32;
  std::unique_ptr<RfftNd<double>> rn64;
  std::unique_ptr<IrfftNd<float>> in32;
  std::unique_ptr<IrfftNd<double>> in64;
  int64_t n = 0, nin = 0, nout = 0;  // element counts (T) per transform
};
}  // namespace

static std::string g_orc_err;
template <template <typename> class PT, typename... A>
static void* plan_direct(int dtype, int64_t n, int D, int scale_mode, A... args) {
  try {
    Handle* h = new Handle();
    h->dtype = dtype; h->kind = 0; h->n = n; h->nin = 2 * n; h->nout = 2 * n;
    try {
      if (dtype == 0) h->p32.reset(new PT<float>(n, D, scale_mode ? 1.0f : default_scale<float>(n, D), args...));
      else h->p64.reset(new PT<double>(n, D, scale_mode ? 1.0 : default_scale<double>(n, D), args...));
    } catch (const std::exception& e) {
      g_orc_err = e.what();
      delete h;
      return nullptr;
    }
    g_orc_err.clear();
    return h;
  } catch (...) { return nullptr; }
}
extern "C" {

void orc_set_vector_bits(int bits) { g_vector_bits = bits; }
int orc_get_vector_bits(void) { return g_vector_bits; }
int orc_max_threads(void) { return Pool::get().size(); }

void* orc_plan_c2c(int dtype, int64_t n, int D, int scale_mode, int nthreads) {
  try {
    Handle* h = new Handle();
    h->dtype = dtype; h->kind = 0; h->n = n; h->nin = 2 * n; h->nout = 2 * n;
    if (dtype == 0) h->p32.reset(anyplan<float>(n, D, scale_mode ? 1.0f : default_scale<float>(n, D), nthreads));
    else h->p64.reset(anyplan<double>(n, D, scale_mode ? 1.0 : default_scale<double>(n, D), nthreads));
    return h;
  } catch (...) { return nullptr; }
}
const char* orc_last_error(void) { return g_orc_err.c_str(); }
void* orc_plan_hvdh(int dtype, int64_t n, int D, int scale_mode, int factors) {
  return plan_direct<HvdhPlan>(dtype, n, D, scale_mode, factors);
}
void* orc_plan_composite(int dtype, int64_t n, int D, int scale_mode) {
  return plan_direct<CompositePlan>(dtype, n, D, scale_mode);
}
void* orc_plan_split(int dtype, int64_t n, int D, int scale_mode) {
  return plan_direct<SplitPlan>(dtype, n, D, scale_mode);
}
int orc_plan_route(void* p) {
  Handle* h = (Handle*)p;
  return h->dtype == 0 ? h->p32->route : h->p64->route;
}
int64_t orc_plan_info(void* p, int64_t* out, int64_t cap) {
  Handle* h = (Handle*)p;
  std::vector<i64> v;
  if (h->dtype == 0) h->p32->info(v); else h->p64->info(v);
  for (int64_t i = 0; i < (int64_t)v.size() && i < cap; ++i) out[i] = v[i];
  return (int64_t)v.size();
}
int orc_execute_c2c(void* p, const void* x, void* y, int64_t batch) {
  Handle* h = (Handle*)p;
  for (int64_t b = 0; b < batch; ++b) {
    if (h->dtype == 0) h->p32->exec((const float*)x + b * h->nin, (float*)y + b * h->nout);
    else h->p64->exec((const double*)x + b * h->nin, (double*)y + b * h->nout);
  }
  return 0;
}
void orc_destroy(void* p) { delete (Handle*)p; }

void* orc_plan_rfft(int dtype, int64_t n, int nthreads) {
  try {
    Handle* h = new Handle();
    h->dtype = dtype; h->kind = 1; h->n = n; h->nin = n; h->nout = 2 * (n / 2 + 1);
    if (dtype == 0) h->r32.reset(new RfftPlan<float>(n, nthreads));
    else h->r64.reset(new RfftPlan<double>(n, nthreads));
    return h;
  } catch (...) { return nullptr; }
}
void* orc_plan_irfft(int dtype, int64_t n, int normalized, int nthreads) {
  try {
    Handle* h = new Handle();
    h->dtype = dtype; h->kind = 2; h->n = n; h->nin = 2 * (n / 2 + 1); h->nout = n;
    if (dtype == 0) h->i32.reset(new IrfftPlan<float>(n, normalized != 0, nthreads));
    else h->i64_.reset(new IrfftPlan<double>(n, normalized != 0, nthreads));
    return h;
  } catch (...) { return nullptr; }
}
int orc_execute_rfft(void* p, const void* x, void* y, int64_t batch) {
  Handle* h = (Handle*)p;
  for (int64_t b = 0; b < batch; ++b) {
    if (h->dtype == 0) h->r32->exec((const float*)x + b * h->nin, (float*)y + b * h->nout);
    else h->r64->exec((const double*)x + b * h->nin, (double*)y + b * h->nout);
  }
  return 0;
}
int orc_execute_irfft(void* p, const void* x, void* y, int64_t batch) {
  Handle* h = (Handle*)p;
  for (int64_t b = 0; b < batch; ++b) {
    if (h->dtype == 0) h->i32->exec((const float*)x + b * h->nin, (float*)y + b * h->nout);
    else h->i64_->exec((const double*)x + b * h->nin, (double*)y + b * h->nout);
  }
  return 0;
}

void* orc_plan_nd(int dtype, int rank, const int64_t* dims, int kind, int nthreads) {
  try {
    std::vector<i64> d(dims, dims + rank);
    i64 len = 1;
    for (i64 v : d) len *= v;
    Handle* h = new Handle();
    h->dtype = dtype; h->kind = 3; h->n = len;
    int D = kind == 0 ? -1 : +1;
    if (dtype == 0) h->p32.reset(new NdPlan<float>(d, D, kind == 1 ? 1.0f / (float)len : 1.0f, nthreads));
    else h->p64.reset(new NdPlan<double>(d, D, kind == 1 ? 1.0 / (double)len : 1.0, nthreads));
    return h;
  } catch (...) { return nullptr; }
}
int orc_execute_nd(void* p, const void* x, void* y) {
  Handle* h = (Handle*)p;
  if (h->dtype == 0) h->p32->exec(x, y); else h->p64->exec(x, y);
  return 0;
}
void* orc_plan_rfft_nd(int dtype, int rank, const int64_t* dims, int nthreads) {
  try {
    std::vector<i64> d(dims, dims + rank);
    Handle* h = new Handle();
    h->dtype = dtype; h->kind = 4;
    if (dtype == 0) h->rn32.reset(new RfftNd<float>(d, nthreads));
    else h->rn64.reset(new RfftNd<double>(d, nthreads));
    return h;
  } catch (...) { return nullptr; }
}
void* orc_plan_irfft_nd(int dtype, int rank, const int64_t* dims, int normalized, int nthreads) {
  try {
    std::vector<i64> d(dims, dims + rank);
    Handle* h = new Handle();
    h->dtype = dtype; h->kind = 5;
    if (dtype == 0) h->in32.reset(new IrfftNd<float>(d, normalized != 0, nthreads));
    else h->in64.reset(new IrfftNd<double>(d, normalized != 0, nthreads));
    return h;
  } catch (...) { return nullptr; }
}
int orc_execute_rfft_nd(void* p, const void* x, void* y) {
  Handle* h = (Handle*)p;
  if (h->dtype == 0) h->rn32->exec((const float*)x, (float*)y); else h->rn64->exec((const double*)x, (double*)y);
  return 0;
}
int orc_execute_irfft_nd(void* p, const void* x, void* y) {
  Handle* h = (Handle*)p;
  if (h->dtype == 0) h->in32->exec((const float*)x, (float*)y); else h->in64->exec((const double*)x, (double*)y);
  return 0;
}
int orc_plan_nd_batched(void* p) {
  Handle* h = (Handle*)p;
  const bool f32 = h->dtype == 0;
  if (h->kind == 3) return (f32 ? ((NdPlan<float>*)h->p32.get())->dim1_batched
                                 : ((NdPlan<double>*)h->p64.get())->dim1_batched) ? 1 : 0;
  if (h->kind == 4) return (f32 ? h->rn32->batched : h->rn64->batched) ? 1 : 0;
  if (h->kind == 5) return (f32 ? h->in32->batched : h->in64->batched) ? 1 : 0;
  return 0;
}

void orc_dft_f64(int64_t n, const double* x, double* y, int sign) { dft_f64(n, x, y, sign); }
double orc_vexp(int dtype, double x) { return dtype == 0 ? (double)vexp<float>((float)x) : vexp<double>(x); }

int orc_factor_radices(int64_t n, int64_t* a, int64_t* primes, int64_t* counts, int64_t cap) {
  Fac f = factor_radices(n);
  if (!f.ok) return -1;
  *a = f.a;
  int64_t k = 0;
  for (auto& pc : f.ps) { if (k < cap) { primes[k] = pc.first; counts[k] = pc.second; } k++; }
  return (int)k;
}
int64_t orc_nextsmooth(int64_t n) { return nextsmooth(n); }
int64_t orc_nextsmooth7(int64_t n) { return nextsmooth7(n); }
int64_t orc_resample_params(int dtype, int64_t n, int64_t* w, double* beta) {
  if (dtype == 0) { RsParts<float> p(n, -1, 1.0f); *w = p.w; *beta = p.beta; return p.m; }
  RsParts<double> p(n, -1, 1.0); *w = p.w; *beta = p.beta; return p.m;
}
}
