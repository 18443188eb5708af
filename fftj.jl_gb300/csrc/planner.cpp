// Host planner and C ABI of the GB300 FFTJ transform library.
//
// The planner restates FFTJ's plan-time work for the GPU: factorization over
// {2, 3, 5, 7, 11, 13} (src/plan.jl:16-45), twiddle tables from FP64
// sincospi with exact angle reduction (src/plan.jl:66-95), the resampling
// parameters and weights of src/resample.jl:9-256, and the real-edge twiddles
// of src/real.jl:26-39. Instead of FFTJ's radix-4/8 stage chain and its
// cache-driven routing between direct chains and four-step, a transform of
// length N is split into the fewest HBM passes whose per-pass radix fits one
// CTA tile (a pass = one Stockham stage of radix R_i, its R_i-point DFT done
// in shared memory by radix-2..16 sub-stages).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "../../include/fftj.h"
#include "fftj_internal.h"
#include "plan_internal.h"

using namespace fftj;
typedef int64_t i64;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

// sin(pi x), cos(pi x) with exact reduction of x to [0, 1/4].
void sincospi(double x, double* s, double* c) {
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
// w_n^e = exp(dir * 2 pi i e / n), exact integer reduction of e mod n
void omega(i64 e, i64 n, int dir, double* re, double* im) {
  i64 r = e % n;
  if (r < 0) r += n;
  double s, c;
  // angle in units of pi: 2 r / n, reduced so that 2r/n in [0, 2)
  sincospi((double)(2 * r) / (double)n, &s, &c);
  *re = c;
  *im = dir * s;
}

bool smooth13(i64 n, std::vector<int>* primes) {
  if (n < 1) return false;
  std::vector<int> ps;
  for (int p : {2, 3, 5, 7, 11, 13})
    while (n % p == 0) { n /= p; ps.push_back(p); }
  if (primes) *primes = ps;
  return n == 1;
}

// ---- resampling parameters (FFTJ src/resample.jl) -------------------------
const int SMOOTH_ODD[7] = {1, 3, 5, 7, 9, 15, 21};
int top_set_bit(i64 x) { return x <= 0 ? 0 : 64 - __builtin_clzll((unsigned long long)x); }
i64 nextsmooth7(i64 N) {  // src/resample.jl:25-31
  for (i64 m = N;; ++m) {
    i64 r = m;
    for (int q : {2, 3, 5, 7})
      while (r % q == 0) r /= q;
    if (r == 1) return m;
  }
}
i64 nextsmooth(i64 N) {  // src/resample.jl:13-21
  i64 best = INT64_MAX;
  for (int o : SMOOTH_ODD) {
    int k = std::max(6, top_set_bit((N + o - 1) / o - 1));
    i64 c = (i64)o << k;
    if (c < best) best = c;
  }
  return best;
}
void gausslegendre(int nq, std::vector<double>& z, std::vector<double>& wq) {  // src/resample.jl:33-53
  z.assign(nq, 0);
  wq.assign(nq, 0);
  const double eps = 2.220446049250313e-16;
  for (int i = 1; i <= nq; ++i) {
    double s, x;
    sincospi((i - 0.25) / (nq + 0.5), &s, &x);
    double dp = 1;
    for (int it = 0; it < 20; ++it) {
      double p0 = 1, p1 = x;
      for (int k = 2; k <= nq; ++k) {
        double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
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
double es_kernel(double z, double beta) {  // src/resample.jl:55
  return std::fabs(z) >= 1 ? 0.0 : std::exp(beta * (std::sqrt(1 - z * z) - 1));
}

struct Resample {
  i64 n, m, w, h;
  double beta;
  std::vector<double> corr;  // scale / (w Phi(j'/m))
  std::vector<double> wt;    // n*w weights
  std::vector<int32_t> l0;   // first grid index per output (unwrapped)
};
// _resample_parts with table weights (src/resample.jl:202-256)
Resample resample_parts(i64 n, bool f64, double scale, i64 m_override = 0) {
  Resample r;
  r.n = n;
  const double epsT = f64 ? 2.220446049250313e-16 : 1.1920928955078125e-07;
  const double tol = 10 * epsT;
  r.m = m_override ? m_override : nextsmooth((i64)std::ceil(2.0 * n));
  const double ratio = std::max((double)n / r.m, 0.5);
  i64 wc = (i64)std::ceil(std::log(1 / tol) / (M_PI * std::sqrt(1 - ratio)));
  r.w = 4 * ((wc + 3) / 4);
  r.beta = 0.97 * M_PI * r.w * (1 - (double)n / (2.0 * r.m));
  r.h = r.w / 2;
  if (g_sched.dry) return r;  // a dry plan needs the sizes, not the tables
  std::vector<double> zq, wq;
  gausslegendre((int)(2 * r.w + 20), zq, wq);
  r.corr.resize(n);
  const i64 hp = (n + 1) / 2;
  for (i64 j = 0; j < n; ++j) {
    const i64 jp = j < hp ? j : j - n;
    const double nu = (double)jp / r.m;
    double Phi = 0;
    for (size_t q = 0; q < zq.size(); ++q) {
      if (!(zq[q] > 0)) continue;
      double s, c;
      sincospi(nu * r.w * zq[q], &s, &c);
      Phi += wq[q] * es_kernel(zq[q], r.beta) * c;
    }
    r.corr[j] = scale / (r.w * Phi);
  }
  r.wt.resize(n * r.w);
  r.l0.resize(n);
  for (i64 k = 0; k < n; ++k) {
    const __int128 km = (__int128)k * r.m;
    const i64 q = (i64)(km / n), rr = (i64)(km % n);
    r.l0[k] = (int32_t)(q - r.h + 1);
    const double delta = (double)rr / n;
    for (i64 i = 0; i < r.w; ++i) r.wt[k * r.w + i] = es_kernel((delta + r.h - 1 - i) / r.h, r.beta);
  }
  return r;
}

// split the prime multiset into k bins with every bin <= rmax (LPT on logs);
// bins sorted descending. Heap-free.
bool split_bins(const int* primes, int np, int k, i64 rmax, i64* bins) {
  int ps[64];
  for (int i = 0; i < np; ++i) ps[i] = primes[i];
  std::sort(ps, ps + np, [](int x, int y) { return x > y; });
  for (int i = 0; i < k; ++i) bins[i] = 1;
  for (int i = 0; i < np; ++i) {
    int best = 0;
    for (int j = 1; j < k; ++j)
      if (bins[j] < bins[best]) best = j;
    bins[best] *= ps[i];
  }
  for (int i = 0; i < k; ++i)
    if (bins[i] > rmax) return false;
  std::sort(bins, bins + k, [](i64 x, i64 y) { return x > y; });
  return true;
}

}  // namespace

namespace fftj {

// ---- Gaussian resampling (Harvey-van der Hoeven), FFTJ src/hvdh.jl -------
// For odd non-smooth n: spread the input with a narrow Gaussian onto a
// smooth t = n + delta coprime to n (permuted so that the length-t transform
// lands row q of the banded system on output q), transform at length t, then
// solve the banded system (band B) for the n unknowns and write them to their
// permuted outputs (src/hvdh.jl:1-19). The GPU solves chunks of L rows with H
// halo rows per side independently, one thread per (batch, chunk), with LU
// factors of every chunk precomputed here in FP64.
i64 gcd_(i64 a, i64 b) {
  while (b) { i64 t = a % b; a = b; b = t; }
  return a < 0 ? -a : a;
}
i64 invmod_(i64 a, i64 m) {  // a^{-1} mod m (gcd(a, m) = 1)
  i64 t = 0, nt = 1, r = m, nr = ((a % m) + m) % m;
  while (nr) {
    const i64 q = r / nr;
    i64 x = t - q * nt; t = nt; nt = x;
    x = r - q * nr; r = nr; nr = x;
  }
  return t < 0 ? t + m : t;
}
i64 fld_(i64 a, i64 b) { i64 q = a / b; if ((a % b != 0) && ((a < 0) != (b < 0))) q--; return q; }

// t coprime to odd n, the smallest o*2^k >= n(1 + 1/128) (src/hvdh.jl:79-92)
i64 hvdh_t(i64 n) {
  const i64 N = (i64)std::ceil(n * (1.0 + 1.0 / 128));
  i64 t = INT64_MAX;
  if (n % 2 == 1) {
    for (int o : {1, 3, 5, 7, 9, 15, 21}) {
      if (gcd_(o, n) != 1) continue;
      int k = 0;
      while (((i64)o << k) < N) k++;
      t = std::min<i64>(t, (i64)o << k);
    }
  } else {
    // even n: the smallest odd 7-smooth length coprime to n
    auto smooth7 = [](i64 m) {
      for (int p : {3, 5, 7})
        while (m % p == 0) m /= p;
      return m == 1;
    };
    for (i64 m = N | 1; m <= 2 * n - 1; m += 2)
      if (smooth7(m) && gcd_(m, n) == 1) { t = m; break; }
  }
  return (t != INT64_MAX && t - n < n) ? t : 0;
}
bool use_hvdh(bool f64, i64 n) { return n % 2 == 1 && n >= (f64 ? 1000 : 16384); }  // src/hvdh.jl:97

// halo rows: the inverse of the band system decays; probe windows of the
// unknown-indexed system and find where a unit right-hand side's solution
// falls below tol (src/hvdh.jl:118-146). Dense Gaussian elimination with
// partial pivoting on (2P+1)^2 systems.
i64 hvdh_halo(i64 n, i64 t, double a, int B, double tol) {
  const double rho = (double)t / n;
  const i64 c = invmod_(t - n, n);
  std::vector<i64> probes;
  const i64 np = std::min<i64>(n, 16);
  for (i64 i = 0; i < np; ++i)
    probes.push_back(np == 1 ? 0 : (i64)std::llround((double)i * (n - 1) / (np - 1)));
  for (i64 h : {n / 2, n / 2 + 1}) probes.push_back((h * c) % n);
  for (i64 P = 64; P <= 512; P *= 2) {
    i64 H = 0;
    const i64 m = 2 * P + 1;
    std::vector<double> M(m * m), rhs(m);
    for (i64 l0 : probes) {
      std::fill(M.begin(), M.end(), 0.0);
      // transpose(M) r = e: build the transpose directly, A[j][i] = M[i][j]
      for (i64 i = 0; i < m; ++i)
        for (i64 j = std::max<i64>(0, i - B - 1); j <= std::min<i64>(m - 1, i + B + 1); ++j) {
          const i64 li = l0 - P + i, lj = l0 - P + j;
          const double d = (double)(t * lj - n * fld_(2 * t * li + n, 2 * n)) / (double)n;
          M[j * m + i] = std::exp(-a * d * d);
        }
      std::fill(rhs.begin(), rhs.end(), 0.0);
      rhs[P] = 1;
      for (i64 k = 0; k < m; ++k) {  // elimination with partial pivoting
        i64 piv = k;
        for (i64 r = k + 1; r < m; ++r)
          if (std::fabs(M[r * m + k]) > std::fabs(M[piv * m + k])) piv = r;
        if (piv != k) {
          for (i64 cc = 0; cc < m; ++cc) std::swap(M[k * m + cc], M[piv * m + cc]);
          std::swap(rhs[k], rhs[piv]);
        }
        const double d = M[k * m + k];
        if (d == 0) continue;
        for (i64 r = k + 1; r < m; ++r) {
          const double f = M[r * m + k] / d;
          if (f == 0) continue;
          for (i64 cc = k; cc < m; ++cc) M[r * m + cc] -= f * M[k * m + cc];
          rhs[r] -= f * rhs[k];
        }
      }
      for (i64 k = m - 1; k >= 0; --k) {
        double v = rhs[k];
        for (i64 cc = k + 1; cc < m; ++cc) v -= M[k * m + cc] * rhs[cc];
        rhs[k] = M[k * m + k] != 0 ? v / M[k * m + k] : 0;
      }
      double mx = 0;
      for (i64 j = 0; j < m; ++j) mx = std::max(mx, std::fabs(rhs[j]));
      for (i64 j = 0; j < m; ++j)
        if (std::fabs(rhs[j]) > tol * mx) H = std::max<i64>(H, std::abs(j - P));
    }
    if (H < P - 2 * B) return (i64)std::ceil(rho * H) + B;
  }
  return -1;
}

constexpr i64 kHvdhTableMax = i64(1) << 30;

struct Hvdh {
  i64 n, t, delta, c, w, h, H, L, R, nchunk;
  int B;
  double alpha, a, b, sc;
  std::vector<double> wt;    // t*w spread weights
  std::vector<int32_t> l0;   // t: first input row of each spread output
  // factor tables row-major across chunks (entry (i, ch) at i*nchunk + ch),
  // so the solve's lanes -- consecutive chunks -- read adjacent entries
  std::vector<double> lf;    // R*nchunk*B forward multipliers (rows i-1 .. i-B)
  std::vector<double> uf;    // R*nchunk*(B+1): 1/U_ii, U_{i,i+1..i+B}
  std::vector<int32_t> oi;   // R*nchunk: output index of the row's unknown (-1: identity row)
  // factors rebuilt in the solve instead (FFTJ factors = :fly): per chunk the
  // column state at its column -B and the output index of its first unknown
  bool fly = false;
  std::vector<int64_t> se, so;
  bool ok = false;
};

Hvdh hvdh_parts(i64 n, bool f64, double scale, i64 nbatch) {
  Hvdh P;
  P.n = n;
  P.t = hvdh_t(n);
  if (!P.t) return P;
  const i64 t = P.t;
  P.delta = t - n;
  P.c = invmod_(P.delta, n);
  P.alpha = f64 ? 1.45 : 1.0;  // src/hvdh.jl:64
  P.a = M_PI * P.alpha * P.alpha;
  P.b = M_PI / (P.alpha * P.alpha);
  const double tol = (f64 ? 2.220446049250313e-16 : 1.1920928955078125e-07) / 4;
  P.h = (i64)std::ceil(P.alpha * std::sqrt(std::log(1 / tol) / M_PI));
  P.w = 2 * P.h;
  P.B = (int)std::floor(std::sqrt(std::log(1 / tol) / P.a) + 0.5);
  if (P.B < 1 || P.B > 3) return P;
  {
    // the probe costs milliseconds; plans of one length (and the tuner's
    // candidates) share its result
    static std::mutex mu;
    static std::map<std::tuple<i64, i64, int, bool>, i64> cache;
    const auto key = std::make_tuple(n, t, P.B, f64);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    P.H = it != cache.end() ? it->second : (cache[key] = hvdh_halo(n, t, P.a, P.B, tol));
  }
  if (P.H < 0) return P;
  // chunks: L rows (a divisor of t), R = L + 2H rows each. The solve runs
  // one thread per (batch, chunk) along a dependent chain of R rows, so L
  // trades halo work (2H / L) for threads: aim for ~40K threads, with L
  // between max(32, 2H) and 128.
  const double want = std::min(128.0, std::max({32.0, 2.0 * (double)P.H, (double)t * nbatch / 40000.0}));
  i64 L = 1;
  for (i64 d = 1; d <= 256; ++d)
    if (t % d == 0 && std::abs((double)d - want) <= std::abs((double)L - want)) L = d;
  P.L = L;
  P.R = L + 2 * P.H;
  P.nchunk = t / L;
  P.sc = scale * (double)n / (double)t;
  // factor tables (8 + 8 B per band entry, 4 B per row) unless they would
  // exceed kHvdhTableMax or the plan asks for factors rebuilt per call.
  // FFTJ caps its tables at 8 MiB (_HVDH_TABLE_MAX, src/hvdh.jl:75) for the
  // CPU's caches; on GB300 the table stream is cheaper than rebuilding
  // (FP64 runs at 1/64 of FP32; 2^20-point primes solve about 2x faster from
  // tables), so the 1 GiB cap only bounds device memory.
  {
    const double tbytes = (double)P.nchunk * P.R * ((2 * P.B + 1) * 8.0 + 4.0);
    P.fly = g_sched.hvdh_factors == 2 || (g_sched.hvdh_factors == 0 && tbytes > (double)kHvdhTableMax);
  }
  if (g_sched.dry) {  // a dry plan needs the sizes, not the tables
    P.ok = true;
    return P;
  }
  // spread table (src/hvdh.jl:726-752 restated per output row)
  const i64 w = P.w, hw = P.h;
  P.wt.resize(t * w);
  P.l0.resize(t);
  for (i64 q = 0; q < t; ++q) {
    const double delta = (double)(t - q) / t;
    for (i64 op = 0; op < w; ++op) {
      const double o = (double)(op + 1 - hw);
      P.wt[q * w + op] = std::exp(-P.b * (delta - o) * (delta - o)) / P.alpha;
    }
    P.l0[q] = (int32_t)((((q * P.c - hw) % n) + n) % n);
  }
  if (P.fly) {
    // per chunk: the column state e = 2 t l' - 2 n q + n at column q0 - B,
    // and Delta l' mod n for the first unknown l' at or after row q0
    // (_hvdh_e, src/hvdh.jl:147-151)
    P.se.resize(P.nchunk);
    P.so.resize(P.nchunk);
    for (i64 ch = 0; ch < P.nchunk; ++ch) {
      const i64 q0 = ((ch * L - P.H) % t + t) % t;
      auto lprime = [&](i64 q) { return -fld_(-(2 * n * q - n), 2 * t); };  // cld(2nq - n, 2t)
      const i64 qb = q0 - P.B;
      const i64 lb = lprime(qb);
      P.se[ch] = 2 * t * lb - 2 * n * qb + n;
      P.so[ch] = (i64)((__int128)P.delta * lprime(q0) % n);
      if (P.so[ch] < 0) P.so[ch] += n;
    }
    P.ok = true;
    return P;
  }
  // rows: hit[q] (an unknown sits nearest row q) and that unknown's index
  std::vector<i64> ell(t, -1);
  for (i64 l = 0; l < n; ++l) {
    const i64 q = fld_(2 * t * l + n, 2 * n);  // nearest row of position rho*l
    ell[((q % t) + t) % t] = l;
  }
  // cyclic distance rho*l - q = (t*l - n*q)/n with an exact integer
  // numerator (rounding rho*l would cost ~1e-13 in the Gaussian entries)
  const i64 nt_ = n * t;
  auto dist = [&](i64 l, i64 q) {
    i64 M = t * l - n * q;
    M = ((M + nt_ / 2) % nt_ + nt_) % nt_ - nt_ / 2;
    return (double)M / (double)n;
  };
  const int B = P.B;
  const i64 R = P.R;
  P.lf.assign(P.nchunk * R * B, 0.0);
  P.uf.assign(P.nchunk * R * (B + 1), 0.0);
  P.oi.assign(P.nchunk * R, -1);
  std::vector<double> A(R * (2 * B + 1));  // band rows: A[i][k], k = col - i + B
  for (i64 ch = 0; ch < P.nchunk; ++ch) {
    const i64 q0 = ch * L - P.H;
    auto qrow = [&](i64 i) { return (((q0 + i) % t) + t) % t; };
    std::fill(A.begin(), A.end(), 0.0);
    for (i64 i = 0; i < R; ++i) {
      const i64 q = qrow(i);
      if (ell[q] < 0) { A[i * (2 * B + 1) + B] = 1.0; continue; }
      P.oi[i * P.nchunk + ch] = (int32_t)((P.delta * ell[q]) % n);
      for (int k = -B; k <= B; ++k) {
        const i64 j = i + k;
        if (j < 0 || j >= R) continue;
        const i64 lj = ell[qrow(j)];
        if (lj < 0) continue;
        const double d = dist(lj, q);
        A[i * (2 * B + 1) + k + B] = std::exp(-P.a * d * d);
      }
    }
    // banded LU without pivoting (src/hvdh.jl:524-566 does it row by row)
    for (i64 i = 0; i < R; ++i) {
      for (int k = B; k >= 1; --k) {
        const i64 j = i - k;  // eliminate column j < i
        if (j < 0) continue;
        const double piv = A[j * (2 * B + 1) + B];
        const double f = A[i * (2 * B + 1) + (j - i) + B] / piv;
        P.lf[(i * P.nchunk + ch) * B + (k - 1)] = f;
        if (f == 0) continue;
        for (int cc = 0; cc <= B; ++cc) {  // row j's U part: columns j .. j+B
          const i64 col = j + cc;
          const int ki = (int)(col - i) + B;
          if (ki < 0 || ki > 2 * B) continue;
          A[i * (2 * B + 1) + ki] -= f * A[j * (2 * B + 1) + B + cc];
        }
      }
      const double d = A[i * (2 * B + 1) + B];
      P.uf[(i * P.nchunk + ch) * (B + 1)] = 1.0 / d;
      for (int j = 1; j <= B; ++j) P.uf[(i * P.nchunk + ch) * (B + 1) + j] = A[i * (2 * B + 1) + B + j];
    }
  }
  P.ok = true;
  return P;
}

// ---- pass decomposition ----
int env_int(const char* name, int dflt) {
  const char* v = std::getenv(name);
  return v && *v ? std::atoi(v) : dflt;
}
thread_local SchedOpts g_sched;

DtypeCfg dtype_cfg(bool f64) {
  // F32: 4096-element tiles (35 KB) give 4 CTAs of 256 threads per SM,
  // measured faster than 8192-element tiles at 2 CTAs per SM. F64: tiles of
  // at most 2048 elements (37 KB) and multi-pass radices of at most 512
  // (>= 4 columns, 64-byte runs, per tile), so that the run-time-radix body's
  // two tile buffers leave two CTAs per SM, in the persistent group kernel
  // too
  DtypeCfg c = f64 ? DtypeCfg{16, env_int("FFTJ_TILE_F64", 2048), 2048, 256, 512, 4}
                   : DtypeCfg{8, env_int("FFTJ_TILE_F32", 4096), 8192, 512, 1024, env_int("FFTJ_MIN_RUN_F32", 8)};
  if (g_sched.tile > 0) c.tile_max = std::min(std::max(g_sched.tile, 256), c.tile_cap);
  if (g_sched.threads_max > 0) c.threads_max = std::min(c.threads_max, std::max(g_sched.threads_max, 64));
  return c;
}


i64 largest_divisor_le(i64 n, i64 cap) {
  if (cap >= n) return n;
  for (i64 d = std::max<i64>(cap, 1); d >= 1; --d)
    if (n % d == 0) return d;
  return 1;
}

// Fewest threads per tile column a pass of radix R needs: every sub-stage's
// butterflies fit the per-thread register budget (max(1, 16/r) butterflies,
// <= 16 elements per thread).
i64 min_threads_per_column(i64 R) {
  int subs[kMaxSub + 4];
  const int ns = sub_radices(R, subs, kMaxSub + 4);
  i64 tf = (R + 15) / 16;
  for (int i = 0; i < ns; ++i) {
    const int r = subs[i];
    if (r <= 1) continue;
    const i64 cap = std::max(1, 16 / r);
    tf = std::max(tf, (R / r + cap - 1) / cap);
  }
  return tf;
}

// Passes of a length-n axis: one pass when the whole transform fits a tile
// and the axis is contiguous; otherwise the fewest passes whose radices keep
// >= min_run contiguous elements per tile row. Heap-free; returns the pass
// count (0: no decomposition within cap passes).
int pass_radices(i64 n, bool f64, bool strided, i64* Rs, int cap) {
  const DtypeCfg cfg = dtype_cfg(f64);
  int primes[64];
  int np = 0;
  i64 r = n;
  for (int p : {2, 3, 5, 7, 11, 13})
    while (r % p == 0 && np < 64) { r /= p; primes[np++] = p; }
  if (r != 1 || n < 1) return 0;
  // one pass holds the whole transform in a tile of <= 16 elements per thread
  const i64 one_cap = std::min<i64>(cfg.tile_cap, 16 * (i64)cfg.threads_max);
  int k = 0;
  if (((!strided && n <= one_cap) || n <= cfg.rmax_multi) && min_threads_per_column(n) <= cfg.threads_max) {
    Rs[0] = n;
    k = 1;
  } else {
    for (int kk = 1; kk <= cap && kk < 16 && !k; ++kk) {
      if (!split_bins(primes, np, kk, cfg.rmax_multi, Rs)) continue;
      bool fits = true;
      for (int i = 0; i < kk; ++i) fits = fits && min_threads_per_column(Rs[i]) <= cfg.threads_max;
      if (fits) k = kk;
    }
    if (!k) return 0;
  }
  // schedule options: more passes than the fewest, then a permutation
  const int want = std::min(std::min(k + std::max(g_sched.extra_passes, 0), cap), std::min(np, 15));
  if (want > k && split_bins(primes, np, want, cfg.rmax_multi, Rs)) k = want;
  if (g_sched.order > 0 && k > 1) {
    // the order-th lexicographic permutation of the (descending) bins
    int idx[16];
    for (int i = 0; i < k; ++i) idx[i] = i;
    int64_t f = 1;
    for (int i = 2; i <= k; ++i) f *= i;
    for (int it = 0; it < (int)(g_sched.order % f); ++it) std::next_permutation(idx, idx + k);
    i64 tmp[16];
    for (int i = 0; i < k; ++i) tmp[i] = Rs[idx[i]];
    for (int i = 0; i < k; ++i) Rs[i] = tmp[i];
  }
  return k;
}

// sub-radix sequence of one pass: odd primes first, then the power-of-two
// part as balanced radix-16/8/4/2 sub-stages (larger first). Returns the count.
int sub_radices(i64 R, int* out, int cap) {
  int k = 0;
  i64 r = R;
  int a = 0;
  while (r % 2 == 0) { r /= 2; a++; }
  for (int p : {3, 5, 7, 11, 13})
    while (r % p == 0 && k < cap) { r /= p; out[k++] = p; }
  if (a > 0) {
    const int parts = (a + 3) / 4;
    const int base = a / parts, extra = a % parts;
    for (int i = 0; i < parts && k < cap; ++i) out[k++] = 1 << (base + (i < extra ? 1 : 0));
  }
  if (k == 0) out[k++] = 1;
  return k;
}

// Everything of a pass but its tables, scale and load op: sub-stages, tile
// (columns of batch x p x q), threads per column, kernel mappings and
// shared memory. Heap-free.
int pass_geometry(PassParams& pp, bool f64, i64 R, i64 m, i64 s, i64 ncur, i64 nbatch, i64 ibs, i64 obs,
                  bool wide) {
  const DtypeCfg cfg = dtype_cfg(f64);
  if (ncur >= ((i64)1 << 31)) return fail(FFTJ_ERR_UNSUPPORTED, "transform length must be below 2^31");
  pp.R = (int)R;
  int subs[kMaxSub + 4];
  const int ns = sub_radices(R, subs, kMaxSub + 4);
  if (ns > kMaxSub) return fail(FFTJ_ERR_UNSUPPORTED, "too many sub-stages");
  pp.nsub = 0;
  i64 S = 1;
  for (int i = 0; i < ns; ++i) {
    const int r = subs[i];
    if (r == 1) continue;
    SubStage& ss = pp.sub[pp.nsub++];
    ss.r = r;
    ss.S = (int)S;
    ss.fS = FastDiv((uint32_t)S);
    ss.Rr = (int)(R / r);
    S *= r;
  }
  pp.m = m;
  pp.s = s;
  pp.ncur = ncur;
  pp.in_bstride = ibs;
  pp.out_bstride = obs;
  pp.nbatch = nbatch;
    // threads per tile column: every sub-stage's butterflies fit the
    // per-thread register budget (max(1, 16/r) butterflies, <= 16 elements)
    auto tf_ok = [&](i64 tf) {
      if ((R + tf - 1) / tf > 16) return false;
      for (int i = 0; i < pp.nsub; ++i) {
        const int r = pp.sub[i].r;
        const i64 cap = std::max(1, 16 / r);
        if ((pp.sub[i].Rr + tf - 1) / tf > cap) return false;
      }
      return true;
    };
    i64 Tf = 1;
    while (!tf_ok(Tf)) Tf++;
    if (g_sched.tf_mult > 1 && Tf * g_sched.tf_mult <= std::min<i64>(R, cfg.threads_max)) Tf *= g_sched.tf_mult;
    // tile: columns (batch, p, q); NB * Tf threads. Passes over strided
    // data keep >= min_run columns (contiguous elements per HBM run).
    const bool one_pass = (m == 1 && s == 1);
    i64 tmax = std::max<i64>(cfg.tile_max, R);
    if (!one_pass) tmax = std::min<i64>(std::max<i64>(tmax, R * cfg.min_run), std::max<i64>(cfg.tile_cap, R));
    i64 cols = std::max<i64>(1, std::min<i64>(tmax / R, cfg.threads_max / Tf));
    if (wide) cols = kWideCols;  // the wide kernel's tile (its own CTA size)
    if (Tf > cfg.threads_max) return fail(FFTJ_ERR_UNSUPPORTED, "pass radix needs too many threads");
    i64 Pt = 1, Qt = 1, NBt = 1;
    if (s == 1) {
      Pt = largest_divisor_le(m, cols);
      if (Pt == m) NBt = std::max<i64>(1, cols / m);
    } else {
      Qt = largest_divisor_le(s, cols);
      // a stride with no good divisor (a large prime factor) gets ragged
      // lane tiles: the last tile's lanes beyond s are masked
      if (Qt * 2 < std::min<i64>(cols, s)) Qt = std::min<i64>(cols, s);
      if (Qt == s) {
        Pt = largest_divisor_le(m, cols / Qt);
        if (Pt == m) NBt = std::max<i64>(1, cols / (m * s));
      }
    }
    NBt = std::min(NBt, nbatch);
    pp.P = (int)Pt;
    pp.Q = (int)Qt;
    pp.NBt = (int)NBt;
    pp.NB = (int)(Pt * Qt * NBt);
    pp.Tf = (int)Tf;
    pp.ept = (int)((R + Tf - 1) / Tf);
    pp.fQ = FastDiv((uint32_t)Qt);
    pp.fP = FastDiv((uint32_t)Pt);
    pp.fR = FastDiv((uint32_t)R);
    pp.fNB = FastDiv((uint32_t)pp.NB);
    pp.tiles_q = (uint32_t)((s + Qt - 1) / Qt);
    pp.tiles_p = (uint32_t)(m / Pt);
    pp.tiles_b = (uint32_t)((nbatch + NBt - 1) / NBt);
    pp.ftq = FastDiv(pp.tiles_q);
    pp.ftp = FastDiv(pp.tiles_p);
    const double ntiles = (double)pp.tiles_q * pp.tiles_p * pp.tiles_b;
    if (ntiles >= 2147483647.0) return fail(FFTJ_ERR_UNSUPPORTED, "grid too large");
    const i64 E = (i64)pp.NB * R;
    pp.threads = (int)(pp.NB * Tf);
    // lanes walk j where the transform axis is contiguous in HBM
    pp.load_rows = (m == 1 && s == 1) ? 1 : 0;
    pp.store_rows = (s == 1) ? 1 : 0;
    if ((pp.load_rows || pp.store_rows) && (E + pp.threads - 1) / pp.threads > 16)
      return fail(FFTJ_ERR_UNSUPPORTED, "tile exceeds 16 elements per thread");
    const int padsh = f64 ? 3 : 4;
    pp.smem_elems = (int)(E + (E >> padsh) + 2);
    // ComplexF64: block fixed point unless the plan asks for FP64 butterflies
    pp.fx = (f64 && !g_sched.f64_arith) ? 1 : 0;
    pp.fx_cols = pp.fx ? pp.NB : 0;
    pp.fx_b0 = 53;  // a pass without sub-stages (R = 1) copies: inputs stay exact
    pp.fx_sht = 0;
    if (pp.fx && pp.nsub > 0) {
      auto lg = [](int r) { int l = 0; while ((1 << l) < r) ++l; return l; };
      pp.fx_b0 = std::min(61 - lg(pp.sub[0].r), 60);
      for (int i = 1; i < pp.nsub; ++i) pp.fx_sht += lg(pp.sub[i].r);
    }
  return FFTJ_OK;
}

// opts.wide_axis: a strided F32 axis of length kWideR runs as one pass of
// kWideCols-column tiles (the kernel built for it has 1024 threads and one
// CTA per SM), so a 2-D 4096 x 4096 transform sweeps HBM twice -- the row
// pass and this column pass -- as FFTJ's Fs2Plan does
// (src/fourstep.jl:500-552), instead of splitting the column transform into
// two passes of 64-point columns. Not the default: its tile rows are 32
// bytes, so each warp's loads and stores touch eight cache lines and the
// pass is bound by the load/store unit (0.37 of HBM on GB300), where the two
// radix-64 passes reach 0.86 each and finish sooner together. Only with the
// tuner's other knobs and the precision form at their defaults, and when
// the kernel exists.
bool wide_axis(bool f64, i64 n, i64 Bi) {
  return g_sched.wide_axis == 1 && !f64 && n == kWideR && Bi > 1 && Bi % kWideCols == 0 && g_sched.precision == 0 &&
         g_sched.extra_passes <= 0 && g_sched.order == 0 && g_sched.tf_mult <= 1 && g_sched.tile == 0 &&
         (g_sched.threads_max == 0 || g_sched.threads_max >= kWideCols * (kWideR / 16));
}

// outer twiddle table layout of a pass: none (last pass), full table
// w_ncur^e, or two-level hi[e >> sh] * lo[e & (2^sh - 1)]
void outer_twiddle_layout(PassParams& pp, bool f64) {
  pp.tw_mode = 0;
  if (pp.m <= 1) return;
  const i64 ncur = pp.ncur;
  // first passes (s == 1) store along j, so their twiddle exponents p*j
  // scatter: F32 reads the small two-level tables (L1-resident) there
  const i64 full_max = f64 ? (1 << 21) : (pp.s == 1 && env_int("FFTJ_TW_FIRST_FULL", 0) == 0 ? 0 : (1 << 22));
  if (ncur <= full_max) {
    pp.tw_mode = 1;
    return;
  }
  int sh = 0;
  while (((i64)1 << (2 * sh)) < ncur) sh++;
  pp.tw_mode = 2;
  pp.tw_shift = sh;
}

// The compile-time recipe kernel matching a pass (same radix sequence, load
// op, direction, threads per column and mapping mode), else nullptr (the
// generic kernel). Heap-free.
template <typename T>
const void* pick_pass_kernel_t(int dir, const PassParams& pp) {
  int count = 0;
  const RecipeEntry* tab = dir < 0 ? recipe_table<T, -1>(&count) : recipe_table<T, 1>(&count);
  int mode = -1;
  if (pp.load_rows && pp.store_rows && (pp.NBt == 1 || pp.out_bstride == (int64_t)pp.R)) mode = 0;
  else if (!pp.load_rows && pp.store_rows && pp.NBt == 1) mode = 1;
  else if (!pp.load_rows && !pp.store_rows) mode = 2;
  // a kernel built for the tile's exact column count first, then any
  for (int want_nb = 1; want_nb >= 0; --want_nb) {
    for (int i = 0; i < count && mode >= 0; ++i) {
      const RecipeEntry& e = tab[i];
      if (e.mode != mode || e.load_op != pp.load_op || e.Tf != pp.Tf) continue;
      if (want_nb ? e.nb != pp.NB : e.nb != 0) continue;
      int n = 0;
      while (n < 6 && e.radix[n]) n++;
      if (n != pp.nsub) continue;
      bool same = true;
      for (int j = 0; j < n; ++j) same = same && e.radix[j] == pp.sub[j].r;
      if (same) return e.fn;
    }
  }
  return nullptr;
}
const void* pick_pass_kernel(bool f64, int dir, const PassParams& pp) {
  // ComplexF64 recipe kernels compute in block fixed point; FP64-butterfly
  // passes run the generic kernel
  if (f64) return pp.fx ? pick_pass_kernel_t<Fx>(dir, pp) : nullptr;
  return pick_pass_kernel_t<float>(dir, pp);
}

// Sub-stage i of a pass runs on the tensor cores in the precision form (the
// host copy of the device condition tc16_fits: whole warps, butterflies in
// n-tiles of 8, at most 4 n-tiles per warp).
bool tc16_substage_fits(const PassParams& pp, int i) {
  const int nbf = pp.NB * pp.sub[i].Rr;
  return pp.sub[i].r == 16 && pp.threads % 32 == 0 && nbf % 8 == 0 && nbf / 8 <= 4 * (pp.threads / 32);
}
bool has_tc16_substage(const PassParams& pp) {
  for (int i = 0; i < pp.nsub; ++i)
    if (tc16_substage_fits(pp, i)) return true;
  return false;
}

// Recipe kernels stage the pass's inner twiddles w_R^t in shared memory
// when the table is small next to the tile; beyond kStageTwiddleMax entries
// they read it from global memory (L1/L2-resident).
constexpr int kStageTwiddleMax = 1024;
// The wide strided pass (one CTA per SM, 1024 threads) stages its 32 KB
// table too (it has the shared memory to spare; 3% faster measured).
bool stage_inner_twiddles(const PassParams& pp, bool recipe) {
  const bool wide = pp.R == kWideR && pp.NB == kWideCols && pp.threads == kWideCols * (kWideR / 16);
  return recipe && (pp.R <= kStageTwiddleMax || wide);
}

void set_error(const char* msg) { g_err = msg; }

}  // namespace fftj

namespace {


}  // namespace

// ---------------------------------------------------------------------------
namespace {

// upload a table of complex values (re, im pairs in double) as T
// Host-built tables of the plan being built on this thread
// (fftj_plan_c2c_from_tables): the roots w_N^e for e < N, and for a
// resampled length the deconvolution and interpolation tables. omega_table
// reads every twiddle table from the roots (n divides N) instead of
// evaluating sincospi.
struct HostTables {
  const double* omega = nullptr;  // 2N values: re, im of w_N^e
  i64 N = 0;
  const fftj_resample_tables_t* rs = nullptr;
};
thread_local HostTables g_tables;

// stand-in address of a table that a dry plan does not build
const void* const kDryTable = reinterpret_cast<const void*>(uintptr_t(256));

template <typename T>
const void* upload_cplx(fftj_plan_s* P, const std::vector<double>& ri) {
  if (g_sched.dry) return kDryTable;
  std::vector<T> h(ri.size());
  for (size_t i = 0; i < ri.size(); ++i) h[i] = (T)ri[i];
  DevBuf b;
  b.bytes = h.size() * sizeof(T);
  if (cudaMalloc(&b.p, std::max<size_t>(b.bytes, 16)) != cudaSuccess) return nullptr;
  if (cudaMemcpy(b.p, h.data(), b.bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(b.p);
    return nullptr;
  }
  P->tables.push_back(b);
  P->table_bytes += b.bytes;
  return b.p;
}
const void* upload_raw(fftj_plan_s* P, const void* data, size_t bytes) {
  if (g_sched.dry) return kDryTable;
  DevBuf b;
  b.bytes = bytes;
  if (cudaMalloc(&b.p, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
  if (cudaMemcpy(b.p, data, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(b.p);
    return nullptr;
  }
  P->tables.push_back(b);
  P->table_bytes += bytes;
  return b.p;
}

// round(c * 2^61) clamped to [-2^61, 2^61 - 1]: the Q61 twiddles of block
// fixed-point passes (fx64.cuh)
int64_t q61(double c) {
  if (c >= 1.0) return ((int64_t)1 << 61) - 1;
  if (c <= -1.0) return -((int64_t)1 << 61);
  return (int64_t)std::llround(c * 2305843009213693952.0);
}
const void* upload_q61(fftj_plan_s* P, const std::vector<double>& ri) {
  if (g_sched.dry) return kDryTable;
  std::vector<int64_t> h(ri.size());
  for (size_t i = 0; i < ri.size(); ++i) h[i] = q61(ri[i]);
  return upload_raw(P, h.data(), h.size() * sizeof(int64_t));
}

// the complex table w_n^e for e in [0, count), sign dir (as T, or as Q61
// integers when as_q61 is set)
template <typename T>
const void* omega_table(fftj_plan_s* P, i64 n, i64 count, i64 stride, int dir, bool as_q61 = false) {
  if (g_sched.dry) return kDryTable;
  std::vector<double> ri(2 * count);
  if (g_tables.omega && g_tables.N % n == 0) {
    // w_n^k = w_N^(k N / n), read from the caller's roots
    const i64 f = g_tables.N / n;
    for (i64 e = 0; e < count; ++e) {
      const i64 k = (i64)(((__int128)e * stride) % n) * f;
      ri[2 * e] = g_tables.omega[2 * k];
      ri[2 * e + 1] = g_tables.omega[2 * k + 1];
    }
  } else {
    for (i64 e = 0; e < count; ++e) omega(e * stride, n, dir, &ri[2 * e], &ri[2 * e + 1]);
  }
  return as_q61 ? upload_q61(P, ri) : upload_cplx<T>(P, ri);
}

// Build the passes of a length-n transform along an axis with inner stride
// Bi (elements between consecutive points of one transform... folded into s)
// for nbatch independent blocks at batch strides ibs/obs. The first pass may
// use a fused load op (filled in by the caller).
template <typename T>
int build_axis_passes(fftj_plan_s* P, i64 n, i64 Bi, i64 nbatch, i64 ibs, i64 obs, int dir, double scale,
                      std::vector<Op>* out_ops) {
  const bool f64 = sizeof(T) == 8;
  i64 Rbuf[16];
  bool wide = wide_axis(f64, n, Bi);
  if (wide) {
    // one pass, if the wide kernel serves its geometry
    PassParams probe;
    std::memset(&probe, 0, sizeof(probe));
    wide = pass_geometry(probe, f64, n, 1, Bi, n, nbatch, ibs, obs, true) == FFTJ_OK &&
           pick_pass_kernel(f64, dir, probe) != nullptr;
  }
  const int npass = wide ? 1 : pass_radices(n, f64, Bi > 1, Rbuf, 16);
  if (wide) Rbuf[0] = n;
  if (npass == 0) return fail(FFTJ_ERR_UNSUPPORTED, "no pass decomposition for length " + std::to_string(n));
  std::vector<i64> Rs(Rbuf, Rbuf + npass);
  i64 s1 = 1;  // 1-D stride before this pass
  i64 ncur = n;
  for (size_t pi = 0; pi < Rs.size(); ++pi) {
    const i64 R = Rs[pi];
    Op op;
    op.kind = OP_PASS;
    op.dir = dir;
    PassParams& pp = op.pp;
    std::memset(&pp, 0, sizeof(pp));
    pp.R = (int)R;
    const i64 m = ncur / R;
    const i64 s = s1 * Bi;  // effective stride
    {
      int grc = pass_geometry(pp, f64, R, m, s, ncur, nbatch, ibs, obs, wide);
      if (grc) return grc;
    }
    // inner twiddles w_R^t (Q61 integers for block fixed-point passes)
    const bool q = pp.fx != 0;
    pp.twR = omega_table<T>(P, R, R, 1, dir, q);
    if (!pp.twR) return fail(FFTJ_ERR_CUDA, "table upload failed");
    // outer twiddles w_ncur^(p*j), p*j < ncur
    outer_twiddle_layout(pp, f64);
    if (pp.tw_mode == 1) {
      pp.tw_full = omega_table<T>(P, ncur, ncur, 1, dir, q);
      if (!pp.tw_full) return fail(FFTJ_ERR_CUDA, "table upload failed");
    } else if (pp.tw_mode == 2) {
      const i64 K = (i64)1 << pp.tw_shift;
      pp.tw_hi = omega_table<T>(P, ncur, (ncur + K - 1) / K, K, dir, q);
      pp.tw_lo = omega_table<T>(P, ncur, K, 1, dir, q);
      if (!pp.tw_hi || !pp.tw_lo) return fail(FFTJ_ERR_CUDA, "table upload failed");
    }
    pp.scale = (pi + 1 == Rs.size()) ? scale : 1.0;
    pp.load_op = LOAD_PLAIN;
    pp.tc = f64 ? 0 : g_sched.precision;
    op.dst_bytes = (size_t)(nbatch * obs) * sizeof(T) * 2;
    out_ops->push_back(op);
    P->pass_R.push_back((int)R);
    s1 *= R;
    ncur /= R;
  }
  return FFTJ_OK;
}

// Chain ops: first reads IN, last writes OUT, intermediates alternate W0/W1.
void wire(std::vector<Op>& ops) {
  const size_t k = ops.size();
  for (size_t i = 0; i < k; ++i) {
    ops[i].src = (i == 0) ? B_IN : ((i - 1) % 2 == 0 ? B_W0 : B_W1);
    ops[i].dst = (i + 1 == k) ? B_OUT : (i % 2 == 0 ? B_W0 : B_W1);
  }
}

int alloc_workspace(fftj_plan_s* P) {
  size_t need[2] = {0, 0};
  for (auto& op : P->ops) {
    if (op.dst == B_W0) need[0] = std::max(need[0], op.dst_bytes);
    if (op.dst == B_W1) need[1] = std::max(need[1], op.dst_bytes);
  }
  // one-op plans that are not in-place safe run through W0 when in == out
  if (P->ops.size() == 1 && !P->inplace_safe) need[0] = std::max(need[0], P->ops[0].dst_bytes);
  for (int i = 0; i < 2; ++i) {
    if (need[i] == 0) continue;
    P->ws[i].bytes = need[i];
    if (P->dry) continue;
    if (cudaMalloc(&P->ws[i].p, need[i]) != cudaSuccess) return fail(FFTJ_ERR_CUDA, "workspace allocation failed");
  }
  return FFTJ_OK;
}

// Gaussian resampling along an axis (hv.n rows, Bi lanes: row r of lane i at
// r Bi + i; nb outer blocks at strides ibs / obs): the spread fused into the
// first pass of the length-t transform, the smooth passes along the axis,
// the chunked banded solve. Bi = 1 is HvdhPlan (src/hvdh.jl:222-241); Bi >
// 1 is the batched HvPass (src/hvdh.jl:696-836), whose lanes share the
// spread weights and the band factors -- on the GPU the lanes are adjacent
// threads of the solve (every lane reads the same factor entry) and the
// axis is chunked as in HvdhPlan, where FFTJ's HvPass factors one cyclic
// chunk per lane vector (same mathematics, more parallelism).
template <typename T>
int build_axis_hvdh(fftj_plan_s* P, const Hvdh& hv, i64 Bi, i64 nb, i64 ibs, i64 obs, int dir,
                    std::vector<Op>* ops) {
  const i64 batch = nb * Bi;  // sequences: outer blocks x lanes
  std::vector<Op> tmp;
  int rc = build_axis_passes<T>(P, hv.t, Bi, nb, Bi * hv.t, Bi * hv.t, dir, 1.0, &tmp);
  if (rc) return rc;
  PassParams& f = tmp.front().pp;
  f.load_op = LOAD_SPREAD;
  f.ld_n = hv.n;
  f.ld_m = hv.t;
  f.ld_stride = ibs;
  f.ld_inner = Bi;
  f.ld_w = (int)hv.w;
  {
    std::vector<T> w(hv.wt.size());
    for (size_t i = 0; i < w.size(); ++i) w[i] = (T)hv.wt[i];
    f.ld_tab = upload_raw(P, w.data(), w.size() * sizeof(T));
    f.ld_l0 = (const int32_t*)upload_raw(P, hv.l0.data(), hv.l0.size() * sizeof(int32_t));
    if (!f.ld_tab || !f.ld_l0) return fail(FFTJ_ERR_CUDA, "table upload failed");
  }
  Op sv;
  sv.kind = OP_SOLVE;
  SolveParams& q = sv.sv;
  std::memset(&q, 0, sizeof(q));
  q.n = hv.n;
  q.t = hv.t;
  q.L = hv.L;
  q.H = hv.H;
  q.R = hv.R;
  q.nchunk = hv.nchunk;
  q.nbatch = batch;
  q.inner = Bi;
  q.g_bstride = Bi * hv.t;
  q.y_bstride = obs;
  q.B = hv.B;
  q.sc = hv.sc;
  q.fly = hv.fly ? 1 : 0;
  q.a = hv.a;
  q.delta = hv.delta;
  if (hv.fly) {
    q.se = (const int64_t*)upload_raw(P, hv.se.data(), hv.se.size() * sizeof(int64_t));
    q.so = (const int64_t*)upload_raw(P, hv.so.data(), hv.so.size() * sizeof(int64_t));
    if (!q.se || !q.so) return fail(FFTJ_ERR_CUDA, "table upload failed");
    // per-thread U rows and output indices of the back pass
    DevBuf ub, ob;
    ub.bytes = (size_t)hv.R * (hv.B + 1) * batch * hv.nchunk * sizeof(T);
    ob.bytes = (size_t)hv.R * batch * hv.nchunk * sizeof(int32_t);
    if (g_sched.dry) {
      ub.bytes = ob.bytes = 0;
      ub.p = ob.p = const_cast<void*>(kDryTable);
    } else if (cudaMalloc(&ub.p, ub.bytes) != cudaSuccess || cudaMalloc(&ob.p, ob.bytes) != cudaSuccess) {
      if (ub.p) cudaFree(ub.p);
      return fail(FFTJ_ERR_CUDA, "workspace allocation failed");
    }
    P->tables.push_back(ub);
    P->tables.push_back(ob);
    q.uw = ub.p;
    q.ow = (int32_t*)ob.p;
  } else {
    std::vector<T> lf(hv.lf.size()), uf(hv.uf.size());
    for (size_t i = 0; i < lf.size(); ++i) lf[i] = (T)hv.lf[i];
    for (size_t i = 0; i < uf.size(); ++i) uf[i] = (T)hv.uf[i];
    q.lf = upload_raw(P, lf.data(), lf.size() * sizeof(T));
    q.uf = upload_raw(P, uf.data(), uf.size() * sizeof(T));
    q.oi = (const int32_t*)upload_raw(P, hv.oi.data(), hv.oi.size() * sizeof(int32_t));
    if (!q.lf || !q.uf || !q.oi) return fail(FFTJ_ERR_CUDA, "table upload failed");
  }
  {
    // forward-substitution scratch owned by the plan
    DevBuf zb;
    zb.bytes = (size_t)hv.R * batch * hv.nchunk * sizeof(T) * 2;
    if (g_sched.dry) zb.bytes = 0, zb.p = const_cast<void*>(kDryTable);
    else if (cudaMalloc(&zb.p, zb.bytes) != cudaSuccess) return fail(FFTJ_ERR_CUDA, "workspace allocation failed");
    P->tables.push_back(zb);
    q.zw = zb.p;
  }
  sv.dst_bytes = (size_t)(nb * obs) * sizeof(T) * 2;
  for (auto& o : tmp) ops->push_back(o);
  ops->push_back(sv);
  P->resample_m = hv.t;
  P->resample_w = hv.w;
  return FFTJ_OK;
}

// HvdH route (src/hvdh.jl:222-241): one lane per batch entry
template <typename T>
int build_c2c_hvdh(fftj_plan_s* P, const Hvdh& hv, i64 batch, i64 idist, i64 odist, int dir,
                   std::vector<Op>* ops, int* route) {
  const int rc = build_axis_hvdh<T>(P, hv, 1, batch, idist, odist, dir, ops);
  if (rc) return rc;
  *route = FFTJ_ROUTE_HVDH;
  return FFTJ_OK;
}

// Split route for non-smooth n = s p with s its 7-smooth part and p odd
// (FFTJ SplitPlan, src/composite.jl:136-301, used here also where FFTJ takes
// CompositePlan): decimate in time, x_r[j] = x[r + s j]; transform the s
// sequences of length p by Gaussian resampling (t ~ 1.008 p, instead of the
// ~2n grid of full-length resampling); multiply output k1 of sequence r by
// w_n^(r k1) in the banded solve; then length-s transforms along r (stride p)
// give X[k1 + p k2] in natural order.
i64 smooth7_part(i64 n) {
  i64 s = 1;
  for (int f : {2, 3, 5, 7})
    while (n % (s * f) == 0) s *= f;
  return s;
}
// FFTJ's thresholds for leaving full-length resampling (src/composite.jl:
// 34-66, 157-161): a sizable smooth part (s >= 16, n >= 4096 F64 / 32768 F32)
// with the odd part Gaussian-resampled from p >= 500 (_COMPOSITE_HV_MINP),
// or a small one (s < 16) for even n >= 16384 F64 / 65536 F32 with an odd
// part FFTJ would route to HvdH. Odd n reach this only below the HvdH
// threshold (full-length HvdH is taken first on the GPU).
bool use_split(bool f64, i64 n) {
  const i64 s = smooth7_part(n), p = n / s;
  if (s < 2 || p % 2 == 0) return false;
  if (g_sched.route == 2) return p >= 64;
  if (g_sched.route != 0) return false;
  if (s >= 16) return n >= (f64 ? 4096 : 32768) && p >= 500;
  return n % 2 == 0 && use_hvdh(f64, p) && n >= (f64 ? 16384 : 65536);
}

template <typename T>
int build_c2c_split(fftj_plan_s* P, i64 n, i64 batch, i64 idist, i64 odist, int dir, double scale,
                    std::vector<Op>* ops, int* route) {
  const i64 s = smooth7_part(n), p = n / s;
  Hvdh hv = hvdh_parts(p, sizeof(T) == 8, 1.0, batch * s);
  if (!hv.ok) return fail(FFTJ_ERR_UNSUPPORTED, "no Gaussian resampling for the odd part");
  Op dec;
  dec.kind = OP_COPY;
  std::memset(&dec.cp, 0, sizeof(dec.cp));
  dec.cp.mode = 5;
  dec.cp.n = n;
  dec.cp.nc = s;
  dec.cp.nbatch = batch;
  dec.cp.in_bstride = idist;
  dec.cp.out_bstride = n;
  dec.dst_bytes = (size_t)(batch * n) * sizeof(T) * 2;
  ops->push_back(dec);
  int r = 0;
  std::vector<Op> hops;
  int rc = build_c2c_hvdh<T>(P, hv, batch * s, p, p, dir, &hops, &r);
  if (rc) return rc;
  SolveParams& sv = hops.back().sv;
  sv.tw = omega_table<T>(P, n, n, 1, dir);
  sv.tw_s = s;
  if (!sv.tw) return fail(FFTJ_ERR_CUDA, "table upload failed");
  for (auto& o : hops) ops->push_back(o);
  std::vector<Op> sops;
  rc = build_axis_passes<T>(P, s, p, batch, n, n, dir, scale, &sops);
  if (rc) return rc;
  sops.back().pp.out_bstride = odist;
  sops.back().dst_bytes = (size_t)(batch * odist) * sizeof(T) * 2;
  for (auto& o : sops) ops->push_back(o);
  P->resample_m = hv.t;
  P->resample_w = hv.w;
  *route = FFTJ_ROUTE_SPLIT;
  return FFTJ_OK;
}

template <typename T>
int build_axis_resample(fftj_plan_s* P, i64 nd, i64 Bi, i64 nb, int dir, double scale, std::vector<Op>* ops);

// FFTJ's CompositePlan (src/composite.jl:10-101): non-smooth n = p s with s
// its 7-smooth part, one Cooley-Tukey step in decimation in frequency (j =
// j1 + p j2, k = k2 + s k1). The length-s transforms over j2 run as the
// passes of an axis of p lanes (exact); a twiddled transpose writes (j1,
// k2) at k2 + s j1 times w_n^(j1 k2); the length-p transforms over j1 are
// one pass along rows j1 with s lanes -- the batched HvPass for p >= 500
// (_COMPOSITE_HV_MINP), batched resampling (RsPass) below -- whose output
// rows k1 of s lanes are already in natural order.
constexpr i64 kCompositeMinS = 16;     // _COMPOSITE_MIN_S
constexpr i64 kCompositeHvMinP = 500;  // _COMPOSITE_HV_MINP
bool use_composite(bool f64, i64 n) {
  const i64 s = smooth7_part(n), p = n / s;
  if (s < 2 || p < 2) return false;
  if (g_sched.route == 4) return true;
  if (g_sched.route != 0) return false;
  return s >= kCompositeMinS && n >= (f64 ? 4096 : 32768);  // _use_composite
}

template <typename T>
int build_c2c_composite(fftj_plan_s* P, i64 n, i64 batch, i64 idist, i64 odist, int dir, double scale,
                        std::vector<Op>* ops, int* route) {
  const bool f64 = sizeof(T) == 8;
  const i64 s = smooth7_part(n), p = n / s;
  std::vector<Op> sops;
  int rc = build_axis_passes<T>(P, s, p, batch, n, n, dir, 1.0, &sops);
  if (rc) return rc;
  sops.front().pp.in_bstride = idist;
  Op tr;
  tr.kind = OP_COPY;
  std::memset(&tr.cp, 0, sizeof(tr.cp));
  tr.cp.mode = 6;
  tr.cp.n = n;
  tr.cp.nc = s;
  tr.cp.nbatch = batch;
  tr.cp.in_bstride = n;
  tr.cp.out_bstride = n;
  tr.cp.tab = omega_table<T>(P, n, n, 1, dir);
  if (!tr.cp.tab) return fail(FFTJ_ERR_CUDA, "table upload failed");
  tr.dst_bytes = (size_t)(batch * n) * sizeof(T) * 2;
  std::vector<Op> pops;
  if (p >= kCompositeHvMinP) {
    Hvdh hv = hvdh_parts(p, f64, scale, batch * s);
    if (!hv.ok) return fail(FFTJ_ERR_UNSUPPORTED, "no Gaussian resampling for the odd part");
    rc = build_axis_hvdh<T>(P, hv, s, batch, n, odist, dir, &pops);
  } else {
    rc = build_axis_resample<T>(P, p, s, batch, dir, scale, &pops);
    if (rc == FFTJ_OK) {
      pops.back().ip.y_bstride = odist;
      pops.back().dst_bytes = (size_t)(batch * odist) * sizeof(T) * 2;
    }
  }
  if (rc) return rc;
  for (auto& o : sops) ops->push_back(o);
  ops->push_back(tr);
  for (auto& o : pops) ops->push_back(o);
  *route = FFTJ_ROUTE_COMPOSITE;
  return FFTJ_OK;
}

// complex 1-D transform of length n (batch at idist/odist) appended to ops;
// if load_op != PLAIN, the first pass uses it with the given parameters.
template <typename T>
int build_c2c_1d(fftj_plan_s* P, i64 n, i64 batch, i64 idist, i64 odist, int dir, double scale,
                 std::vector<Op>* ops, int* route) {
  std::vector<int> primes;
  const bool smooth = smooth13(n, &primes);
  // opts.route = 3: Gaussian resampling at full length for any length, as
  // FFTJ._hvdh (src/hvdh.jl:153-209) is built directly; FFTJ throws
  // ArgumentError when no smooth t is coprime to n (src/hvdh.jl:160-161)
  if (g_sched.route == 3 && !g_tables.rs && n >= 2) {
    Hvdh hv = hvdh_parts(n, sizeof(T) == 8, scale, batch);
    if (!hv.t) return fail(FFTJ_ERR_ARG, "no coprime smooth t for n = " + std::to_string(n));
    if (hv.ok) return build_c2c_hvdh<T>(P, hv, batch, idist, odist, dir, ops, route);
  }
  if (smooth) {
    // intermediate passes use dense strides n
    std::vector<Op> tmp;
    int rc = build_axis_passes<T>(P, n, 1, batch, n, n, dir, scale, &tmp);
    if (rc) return rc;
    tmp.front().pp.in_bstride = idist;
    tmp.back().pp.out_bstride = odist;
    tmp.back().dst_bytes = (size_t)(batch * odist) * sizeof(T) * 2;
    *route = tmp.size() > 1 ? FFTJ_ROUTE_FOURSTEP : FFTJ_ROUTE_DIRECT;
    for (auto& o : tmp) ops->push_back(o);
    return FFTJ_OK;
  }
  // FFTJ's _anyplan tries CompositePlan first (src/plan.jl:196)
  if (!g_tables.rs && use_composite(sizeof(T) == 8, n)) {
    const size_t mark = ops->size();
    const int rc = build_c2c_composite<T>(P, n, batch, idist, odist, dir, scale, ops, route);
    if (rc == FFTJ_OK) return rc;
    ops->resize(mark);  // fall back to the next route
  }
  // odd non-smooth lengths FFTJ sends to Gaussian resampling (HvdH)
  const bool hv_ok = !g_tables.rs && (g_sched.route == 2 ? (n % 2 == 1 && n >= 64)
                                                         : (g_sched.route == 0 && use_hvdh(sizeof(T) == 8, n)));
  if (hv_ok) {
    Hvdh hv = hvdh_parts(n, sizeof(T) == 8, scale, batch);
    if (hv.ok) return build_c2c_hvdh<T>(P, hv, batch, idist, odist, dir, ops, route);
  }
  // even non-smooth lengths whose odd part FFTJ would Gaussian-resample
  if (!g_tables.rs && use_split(sizeof(T) == 8, n)) {
    const size_t mark = ops->size();
    const int rc = build_c2c_split<T>(P, n, batch, idist, odist, dir, scale, ops, route);
    if (rc == FFTJ_OK) return rc;
    ops->resize(mark);  // fall back to full-length resampling
  }
  // non-smooth: resample onto m (src/resample.jl:258-276), from the caller's
  // tables when it supplied them
  Resample rs;
  if (g_tables.rs) {
    const fftj_resample_tables_t* t = g_tables.rs;
    rs.n = n;
    rs.m = t->m;
    rs.w = t->w;
    rs.h = t->w / 2;
    rs.beta = 0;
    rs.corr.assign(t->corr, t->corr + n);
    rs.wt.assign(t->wt, t->wt + n * t->w);
    rs.l0.assign(t->l0, t->l0 + n);
  } else {
    rs = resample_parts(n, sizeof(T) == 8, scale);
  }
  P->resample_m = rs.m;
  P->resample_w = rs.w;
  std::vector<Op> tmp;
  int rc = build_axis_passes<T>(P, rs.m, 1, batch, rs.m, rs.m, dir, 1.0, &tmp);
  if (rc) return rc;
  PassParams& f = tmp.front().pp;
  f.load_op = LOAD_DECONV;
  f.ld_n = n;
  f.ld_m = rs.m;
  f.ld_hp = (n + 1) / 2;
  f.ld_stride = idist;
  f.ld_inner = 1;
  {
    std::vector<T> c(rs.corr.size());  // empty in a dry plan
    for (size_t j = 0; j < c.size(); ++j) c[j] = (T)rs.corr[j];
    f.ld_tab = upload_raw(P, c.data(), c.size() * sizeof(T));
    if (!f.ld_tab) return fail(FFTJ_ERR_CUDA, "table upload failed");
  }
  Op ip;
  ip.kind = OP_INTERP;
  ip.ip.n = n;
  ip.ip.m = rs.m;
  ip.ip.w = rs.w;
  ip.ip.nbatch = batch;
  ip.ip.g_bstride = rs.m;
  ip.ip.y_bstride = odist;
  ip.ip.inner = 1;
  {
    std::vector<T> w(rs.wt.size());
    for (size_t i = 0; i < w.size(); ++i) w[i] = (T)rs.wt[i];
    ip.ip.wt = upload_raw(P, w.data(), w.size() * sizeof(T));
    ip.ip.l0 = (const int32_t*)upload_raw(P, rs.l0.data(), rs.l0.size() * sizeof(int32_t));
    if (!ip.ip.wt || !ip.ip.l0) return fail(FFTJ_ERR_CUDA, "table upload failed");
  }
  ip.dst_bytes = (size_t)(batch * odist) * sizeof(T) * 2;
  for (auto& o : tmp) ops->push_back(o);
  ops->push_back(ip);
  *route = FFTJ_ROUTE_RESAMPLE;
  return FFTJ_OK;
}

// A non-smooth N-d axis (length nd, inner stride Bi, nb outer blocks) by
// batched resampling (FFTJ RsPass, src/resample.jl:434-588, with
// m = nextsmooth7(2 nd) and table weights; _rs_pass!, src/ndplan.jl:137-151):
// the deconvolving first pass writes an m-row grid per block, the smooth
// passes transform it along the axis, the interpolation writes nd rows back.
// scale is folded into the deconvolution.
template <typename T>
int build_axis_resample(fftj_plan_s* P, i64 nd, i64 Bi, i64 nb, int dir, double scale, std::vector<Op>* ops) {
  Resample rs = resample_parts(nd, sizeof(T) == 8, scale, nextsmooth7(2 * nd));
  std::vector<Op> tmp;
  int rc = build_axis_passes<T>(P, rs.m, Bi, nb, Bi * rs.m, Bi * rs.m, dir, 1.0, &tmp);
  if (rc) return rc;
  PassParams& f = tmp.front().pp;
  f.load_op = LOAD_DECONV;
  f.ld_n = nd;
  f.ld_m = rs.m;
  f.ld_hp = (nd + 1) / 2;
  f.ld_stride = Bi * nd;
  f.ld_inner = Bi;
  {
    std::vector<T> c(rs.corr.size());  // empty in a dry plan
    for (size_t j = 0; j < c.size(); ++j) c[j] = (T)rs.corr[j];
    f.ld_tab = upload_raw(P, c.data(), c.size() * sizeof(T));
    if (!f.ld_tab) return fail(FFTJ_ERR_CUDA, "table upload failed");
  }
  Op ip;
  ip.kind = OP_INTERP;
  ip.ip.n = nd;
  ip.ip.m = rs.m;
  ip.ip.w = rs.w;
  ip.ip.nbatch = nb;
  ip.ip.g_bstride = Bi * rs.m;
  ip.ip.y_bstride = Bi * nd;
  ip.ip.inner = Bi;
  {
    std::vector<T> w(rs.wt.size());
    for (size_t i = 0; i < w.size(); ++i) w[i] = (T)rs.wt[i];
    ip.ip.wt = upload_raw(P, w.data(), w.size() * sizeof(T));
    ip.ip.l0 = (const int32_t*)upload_raw(P, rs.l0.data(), rs.l0.size() * sizeof(int32_t));
    if (!ip.ip.wt || !ip.ip.l0) return fail(FFTJ_ERR_CUDA, "table upload failed");
  }
  ip.dst_bytes = (size_t)(nb * Bi * nd) * sizeof(T) * 2;
  for (auto& o : tmp) ops->push_back(o);
  ops->push_back(ip);
  return FFTJ_OK;
}

template <typename T>
int plan_c2c_t(fftj_plan_s* P, const std::vector<i64>& dims, i64 batch, i64 idist, i64 odist, int dir,
               double scale) {
  const i64 len = P->n;
  if (dims.size() == 1) {
    int route = 0;
    int rc = build_c2c_1d<T>(P, len, batch, idist, odist, dir, scale, &P->ops, &route);
    if (rc) return rc;
    P->route = route;
  } else {
    if (idist != len || odist != len)
      return fail(FFTJ_ERR_UNSUPPORTED, "N-d plans need dense batches (idist = odist = prod(dims))");
    P->route = FFTJ_ROUTE_ND;
    // per-dim passes (src/ndplan.jl:57-118), dims of length 1 skipped
    std::vector<size_t> active;
    for (size_t d = 0; d < dims.size(); ++d)
      if (dims[d] > 1) active.push_back(d);
    for (size_t ai = 0; ai < active.size(); ++ai) {
      const size_t d = active[ai];
      const i64 nd = dims[d];
      i64 Bi = 1, Bo = 1;
      for (size_t e = 0; e < d; ++e) Bi *= dims[e];
      for (size_t e = d + 1; e < dims.size(); ++e) Bo *= dims[e];
      const bool last = ai + 1 == active.size();
      int rc = smooth13(nd, nullptr)
                   ? build_axis_passes<T>(P, nd, Bi, Bo * batch, Bi * nd, Bi * nd, dir, last ? scale : 1.0, &P->ops)
                   : build_axis_resample<T>(P, nd, Bi, Bo * batch, dir, last ? scale : 1.0, &P->ops);
      if (rc) return rc;
    }
    if (P->ops.empty()) {
      // all dims 1: y = scale * x as a single radix-1 pass
      return fail(FFTJ_ERR_UNSUPPORTED, "all dimensions have length 1");
    }
  }
  return FFTJ_OK;
}

// rfft (src/real.jl:41-52, 80-142) along dim 1, batched over nb pencils
template <typename T>
int build_r2c_1d(fftj_plan_s* P, i64 n, i64 nb, i64 idist, i64 odist, std::vector<Op>* ops, int* route) {
  const i64 h = n / 2;
  if (n % 2 == 0 && idist % 2 == 0) {
    std::vector<Op> inner;
    int rc = build_c2c_1d<T>(P, h, nb, idist / 2, h, -1, 1.0, &inner, route);
    if (rc) return rc;
    Op post;
    post.kind = OP_RPOST;
    post.rp.h = h;
    post.rp.nbatch = nb;
    post.rp.z_bstride = h;
    post.rp.y_bstride = odist;
    // twiddles w_n^k for k <= h/2 (the mirror's is -conj(w^k)): one table,
    // or for long halves hi[k >> sh] lo[k & (2^sh - 1)] from two small
    // tables (a table of h/2 entries would stream from HBM beside the data)
    const i64 nk = h / 2 + 1;
    post.rp.sh = 0;
    post.rp.tw2 = nullptr;
    if (nk > (1 << 16)) {
      int sh = 0;
      while (((i64)1 << (2 * sh)) < nk) sh++;
      const i64 K = (i64)1 << sh, nh = (nk + K - 1) / K;
      std::vector<double> hi(2 * nh), lo(2 * K);
      for (i64 u = 0; u < nh; ++u) omega(u * K, n, -1, &hi[2 * u], &hi[2 * u + 1]);
      for (i64 t = 0; t < K; ++t) omega(t, n, -1, &lo[2 * t], &lo[2 * t + 1]);
      post.rp.tw = upload_cplx<T>(P, hi);
      post.rp.tw2 = upload_cplx<T>(P, lo);
      if (!post.rp.tw2) return fail(FFTJ_ERR_CUDA, "table upload failed");
      post.rp.sh = sh;
    } else {
      std::vector<double> tw(2 * nk);
      for (i64 k = 0; k < nk; ++k) omega(k, n, -1, &tw[2 * k], &tw[2 * k + 1]);
      post.rp.tw = upload_cplx<T>(P, tw);
    }
    if (!post.rp.tw) return fail(FFTJ_ERR_CUDA, "table upload failed");
    post.dst_bytes = (size_t)(nb * odist) * sizeof(T) * 2;
    for (auto& o : inner) ops->push_back(o);
    ops->push_back(post);
    return FFTJ_OK;
  }
  // odd n: full complex transform (src/real.jl:136-140)
  Op cvt;
  cvt.kind = OP_COPY;
  cvt.cp.mode = 0;
  cvt.cp.n = n;
  cvt.cp.nbatch = nb;
  cvt.cp.in_bstride = idist;
  cvt.cp.out_bstride = n;
  cvt.dst_bytes = (size_t)(nb * n) * sizeof(T) * 2;
  ops->push_back(cvt);
  std::vector<Op> inner;
  int rc = build_c2c_1d<T>(P, n, nb, n, n, -1, 1.0, &inner, route);
  if (rc) return rc;
  for (auto& o : inner) ops->push_back(o);
  Op tr;
  tr.kind = OP_COPY;
  tr.cp.mode = 3;
  tr.cp.n = h + 1;
  tr.cp.nbatch = nb;
  tr.cp.in_bstride = n;
  tr.cp.out_bstride = odist;
  tr.dst_bytes = (size_t)(nb * odist) * sizeof(T) * 2;
  ops->push_back(tr);
  return FFTJ_OK;
}

// irfft / brfft (src/real.jl:57-73, 144-211) along dim 1, nb pencils
template <typename T>
int build_c2r_1d(fftj_plan_s* P, i64 n, i64 nb, i64 idist, i64 odist, bool normalized, double extra_scale,
                 std::vector<Op>* ops, int* route) {
  const i64 h = n / 2;
  if (n % 2 == 0 && odist % 2 == 0) {
    std::vector<Op> inner;
    const double sc = (normalized ? 1.0 / (double)h : 1.0) * extra_scale;
    int rc = build_c2c_1d<T>(P, h, nb, h, odist / 2, +1, sc, &inner, route);
    if (rc) return rc;
    PassParams& f = inner.front().pp;
    const bool fused = inner.front().kind == OP_PASS && f.load_op == LOAD_PLAIN;
    // the pre-pass twiddles w_n^k, k < h: one table, or for a fused pre-pass
    // of a long half hi[k >> sh] lo[k & (2^sh - 1)] from two small tables
    // (an h-entry table would stream from HBM beside the data)
    const void* twd = nullptr;
    const void* twd_lo = nullptr;
    int sh = 0;
    if (fused && h > (1 << 16)) {
      while (((i64)1 << (2 * sh)) < h) sh++;
      const i64 K = (i64)1 << sh, nh = (h + K - 1) / K;
      std::vector<double> hi(2 * nh), lo(2 * K);
      for (i64 u = 0; u < nh; ++u) omega(u * K, n, +1, &hi[2 * u], &hi[2 * u + 1]);
      for (i64 t = 0; t < K; ++t) omega(t, n, +1, &lo[2 * t], &lo[2 * t + 1]);
      twd = upload_cplx<T>(P, hi);
      twd_lo = upload_cplx<T>(P, lo);
      if (!twd || !twd_lo) return fail(FFTJ_ERR_CUDA, "table upload failed");
    } else {
      std::vector<double> tw(2 * h);
      for (i64 k = 0; k < h; ++k) omega(k, n, +1, &tw[2 * k], &tw[2 * k + 1]);
      twd = upload_cplx<T>(P, tw);
      if (!twd) return fail(FFTJ_ERR_CUDA, "table upload failed");
    }
    if (fused) {
      // the pre-pass rides on the first pass's loads
      f.load_op = LOAD_C2R_PRE;
      f.ld_n = h;
      f.ld_stride = idist;
      f.ld_tab = twd;
      f.ld_tab2 = twd_lo;
      f.ld_sh = sh;
      f.ld_pre = normalized ? 0.5 : 1.0;
      f.ld_tab3 = nullptr;
      if (f.m > 1 && f.s == 1) {
        // first pass of several: entry g = p + t m takes w_n^g = w_n^p w_2R^t
        // (R-entry table; the column factor from the tables above)
        std::vector<double> tr(2 * f.R);
        for (i64 t = 0; t < f.R; ++t) omega(t * f.m, n, +1, &tr[2 * t], &tr[2 * t + 1]);
        f.ld_tab3 = upload_cplx<T>(P, tr);
        if (!f.ld_tab3) return fail(FFTJ_ERR_CUDA, "table upload failed");
      }
      for (auto& o : inner) ops->push_back(o);
      return FFTJ_OK;
    }
    // resampled half length: a separate pre-pass feeds the inner transform
    std::vector<Op> inner2;
    rc = build_c2c_1d<T>(P, h, nb, h, odist / 2, +1, sc, &inner2, route);
    if (rc) return rc;
    Op pre;
    pre.kind = OP_COPY;
    pre.cp.mode = 4;
    pre.cp.n = h;
    pre.cp.nbatch = nb;
    pre.cp.in_bstride = idist;
    pre.cp.out_bstride = h;
    pre.cp.tab = twd;
    pre.cp.pre = normalized ? 0.5 : 1.0;
    pre.dst_bytes = (size_t)(nb * h) * sizeof(T) * 2;
    ops->push_back(pre);
    for (auto& o : inner2) ops->push_back(o);
    return FFTJ_OK;
  }
  // odd n: Hermitian expansion, full complex inverse, real part
  Op ex;
  ex.kind = OP_COPY;
  ex.cp.mode = 1;
  ex.cp.n = n;
  ex.cp.nc = h + 1;
  ex.cp.nbatch = nb;
  ex.cp.in_bstride = idist;
  ex.cp.out_bstride = n;
  ex.dst_bytes = (size_t)(nb * n) * sizeof(T) * 2;
  ops->push_back(ex);
  std::vector<Op> inner;
  const double sc = (normalized ? 1.0 / (double)n : 1.0) * extra_scale;
  int rc = build_c2c_1d<T>(P, n, nb, n, n, +1, sc, &inner, route);
  if (rc) return rc;
  for (auto& o : inner) ops->push_back(o);
  Op re;
  re.kind = OP_COPY;
  re.cp.mode = 2;
  re.cp.n = n;
  re.cp.nbatch = nb;
  re.cp.in_bstride = n;
  re.cp.out_bstride = odist;
  re.dst_bytes = (size_t)(nb * odist) * sizeof(T);
  ops->push_back(re);
  return FFTJ_OK;
}

template <typename T>
int plan_r2c_t(fftj_plan_s* P, const std::vector<i64>& dims, i64 batch, i64 idist, i64 odist) {
  const i64 n1 = dims[0];
  const i64 h1p = n1 / 2 + 1;
  i64 rest = 1;
  for (size_t d = 1; d < dims.size(); ++d) rest *= dims[d];
  int route = 0;
  if (dims.size() == 1) {
    int rc = build_r2c_1d<T>(P, n1, batch, idist, odist, &P->ops, &route);
    if (rc) return rc;
    P->route = route;
    return FFTJ_OK;
  }
  if (idist != P->n || odist != h1p * rest)
    return fail(FFTJ_ERR_UNSUPPORTED, "N-d real plans need dense batches");
  P->route = FFTJ_ROUTE_ND;
  // dim-1 real edge per pencil, then complex passes over dims 2..N
  // (src/ndplan.jl:369-427)
  int rc = build_r2c_1d<T>(P, n1, rest * batch, n1, h1p, &P->ops, &route);
  if (rc) return rc;
  std::vector<i64> cd(dims);
  cd[0] = h1p;
  for (size_t d = 1; d < dims.size(); ++d) {
    if (dims[d] == 1) continue;
    i64 Bi = 1, Bo = 1;
    for (size_t e = 0; e < d; ++e) Bi *= cd[e];
    for (size_t e = d + 1; e < cd.size(); ++e) Bo *= cd[e];
    rc = smooth13(dims[d], nullptr)
             ? build_axis_passes<T>(P, dims[d], Bi, Bo * batch, Bi * dims[d], Bi * dims[d], -1, 1.0, &P->ops)
             : build_axis_resample<T>(P, dims[d], Bi, Bo * batch, -1, 1.0, &P->ops);
    if (rc) return rc;
  }
  return FFTJ_OK;
}

template <typename T>
int plan_c2r_t(fftj_plan_s* P, const std::vector<i64>& dims, i64 batch, i64 idist, i64 odist, bool normalized) {
  const i64 n1 = dims[0];
  const i64 h1p = n1 / 2 + 1;
  i64 rest = 1;
  for (size_t d = 1; d < dims.size(); ++d) rest *= dims[d];
  int route = 0;
  if (dims.size() == 1) {
    int rc = build_c2r_1d<T>(P, n1, batch, idist, odist, normalized, 1.0, &P->ops, &route);
    if (rc) return rc;
    P->route = route;
    return FFTJ_OK;
  }
  if (odist != P->n || idist != h1p * rest)
    return fail(FFTJ_ERR_UNSUPPORTED, "N-d real plans need dense batches");
  P->route = FFTJ_ROUTE_ND;
  // complex backward passes over dims 2..N, then the dim-1 real edge
  // (src/ndplan.jl:455-519); normalization folded into the last op
  std::vector<i64> cd(dims);
  cd[0] = h1p;
  for (size_t d = 1; d < dims.size(); ++d) {
    if (dims[d] == 1) continue;
    i64 Bi = 1, Bo = 1;
    for (size_t e = 0; e < d; ++e) Bi *= cd[e];
    for (size_t e = d + 1; e < cd.size(); ++e) Bo *= cd[e];
    int rc = smooth13(dims[d], nullptr)
                 ? build_axis_passes<T>(P, dims[d], Bi, Bo * batch, Bi * dims[d], Bi * dims[d], +1, 1.0, &P->ops)
                 : build_axis_resample<T>(P, dims[d], Bi, Bo * batch, +1, 1.0, &P->ops);
    if (rc) return rc;
  }
  const double extra = normalized ? 1.0 / (double)rest : 1.0;
  return build_c2r_1d<T>(P, n1, rest * batch, h1p, n1, normalized, extra, &P->ops, &route);
}

int check_dims(int rank, const int64_t* dims, std::vector<i64>* out) {
  if (rank < 1 || !dims) return fail(FFTJ_ERR_ARG, "rank must be >= 1");
  out->assign(dims, dims + rank);
  for (i64 d : *out)
    if (d < 1) return fail(FFTJ_ERR_ARG, "transform length must be positive (got " + std::to_string(d) + ")");
  return FFTJ_OK;
}

// Pick the compile-time recipe kernel matching a pass (same radix sequence,
// load op, direction and threads per column), else the generic kernel, and
// opt it into its shared memory.
// Pick each pass's kernel (compile-time recipe or generic) and opt it into
// its shared memory.
// The pipelined tensor-copy kernel of an F32 pass, when the pass's tile is
// a box of its input tensor: columns contiguous in HBM row by row (first
// passes: P columns p, one batch entry; later passes: Q columns q, P = 1,
// one batch entry), an even column count (16-byte box rows) and even
// strides (16-byte tensor strides). The source address is checked at launch.
void pick_tma(Op& op, bool dry) {
  const PassParams& pp = op.pp;
  if (pp.load_op != LOAD_PLAIN) return;
  int mode = -1;
  if (pp.load_rows && pp.store_rows && pp.P == 1 && pp.Q == 1 && (pp.NBt == 1 || pp.out_bstride == (int64_t)pp.R)) {
    // single pass over whole transforms: one 1-D bulk copy per batch entry
    // (R contiguous elements, 16-byte aligned when R and the batch stride
    // are even)
    mode = 0;
    if (pp.R % 2 || (pp.nbatch > 1 && pp.in_bstride % 2)) return;
  } else if (pp.NBt != 1) {
    return;
  } else if (!pp.load_rows && pp.store_rows && pp.Q == 1) {
    mode = 1;
  } else if (!pp.load_rows && !pp.store_rows && pp.P == 1) {
    mode = 2;
  }
  if (mode < 0) return;
  const i64 cols = mode == 1 ? pp.P : mode == 2 ? pp.Q : 2;
  if (mode && (cols != pp.NB || cols % 2 || cols > 256)) return;
  // the last pass of a two-sub-stage radix with 128-byte tile rows keeps
  // plain loads: its in-CTA work is short, and four one-tile CTAs per SM
  // keep more reads in flight than three pipelined ones (measured on the
  // radix-256 last passes of 2^26 and 2^25 x 4: 0.92-0.96 vs 0.84-0.87 of HBM)
  if (pp.m == 1 && pp.nsub == 2 && cols * 8 <= 128) return;
  if (mode && (mode == 1 ? pp.m : pp.s) % 2) return;
  if (pp.nbatch > 1 && (pp.in_bstride % 2 || pp.in_bstride < pp.ncur)) return;
  // the precision form (FP16 hi + lo) has tensor-core variants of these
  // kernels; its BF16 form keeps the run-time kernel
  if (pp.tc > 1) return;
  int count = 0;
  const RecipeEntry* tab = pp.tc ? tma_tc_table(&count) : tma_table(op.dir, &count);
  const void* fn = nullptr;
  for (int i = 0; i < count && !fn; ++i) {
    const RecipeEntry& e = tab[i];
    if (e.dir != op.dir || e.mode != mode || e.nb != pp.NB || e.Tf != pp.Tf || e.tc != pp.tc) continue;
    int n = 0;
    while (n < 6 && e.radix[n]) n++;
    bool same = n == pp.nsub;
    for (int j = 0; j < n && same; ++j) same = e.radix[j] == pp.sub[j].r;
    if (same) fn = e.fn;
  }
  if (!fn) return;
  op.pp.tma_rows = (int)largest_divisor_le(pp.R, 256);
  op.pp.tma_buf = (pp.smem_elems + 15) / 16 * 16;
  op.pp.tma_wait_ns = 1000000000ull;
  op.pp.tma_extra_tx = 0;
  if (!dry) {
    op.tma_grid = tma_prepare(fn, op.pp);
    if (op.tma_grid <= 0) return;
  }
  op.kfn_tma = fn;
  op.tma_mode = mode;
  op.tmap_src = nullptr;
}

using TensorEncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

TensorEncodeFn tensor_encode_fn() {
  static TensorEncodeFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (TensorEncodeFn) nullptr;
    return (TensorEncodeFn)p;
  }();
  return fn;
}

// Tensor map of a pipelined pass's input at `src` (8-byte complex elements
// copied as opaque 64-bit words): first passes (p, j, batch), later passes
// (q, p, j, batch); boxes of one tile's columns x tma_rows rows.
bool encode_tma(Op& op, const void* src) {
  const TensorEncodeFn enc = tensor_encode_fn();
  if (!enc) return false;
  const PassParams& pp = op.pp;
  const cuuint64_t bstr = (cuuint64_t)(pp.nbatch > 1 ? pp.in_bstride : pp.ncur) * 8;
  cuuint64_t dims[4], strides[3];
  cuuint32_t box[4], es[4] = {1, 1, 1, 1};
  cuuint32_t rank;
  if (op.tma_mode == 1) {
    rank = 3;
    dims[0] = (cuuint64_t)pp.m; dims[1] = (cuuint64_t)pp.R; dims[2] = (cuuint64_t)pp.nbatch;
    strides[0] = (cuuint64_t)pp.m * 8; strides[1] = bstr;
    box[0] = (cuuint32_t)pp.P; box[1] = (cuuint32_t)pp.tma_rows; box[2] = 1;
  } else {
    rank = 4;
    dims[0] = (cuuint64_t)pp.s; dims[1] = (cuuint64_t)pp.m; dims[2] = (cuuint64_t)pp.R; dims[3] = (cuuint64_t)pp.nbatch;
    strides[0] = (cuuint64_t)pp.s * 8; strides[1] = (cuuint64_t)(pp.m * pp.s) * 8; strides[2] = bstr;
    box[0] = (cuuint32_t)pp.Q; box[1] = 1; box[2] = (cuuint32_t)pp.tma_rows; box[3] = 1;
  }
  return enc(&op.tmap, CU_TENSOR_MAP_DATA_TYPE_UINT64, rank, const_cast<void*>(src), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <typename T>
int finalize_passes(fftj_plan_s* P) {
  P->plain_loads = g_sched.plain_loads;
  bool any_tma = false;
  for (auto& op : P->ops) {
    if (op.kind != OP_PASS) continue;
    // the precision form's tensor-core sub-stage lives in the run-time
    // kernel; passes without a radix-16 sub-stage keep their recipe kernel
    if (op.pp.tc && !has_tc16_substage(op.pp)) op.pp.tc = 0;
    op.kfn = op.pp.tc ? nullptr : pick_pass_kernel(sizeof(T) == 8, op.dir, op.pp);
    if (!op.kfn && !op.pp.tc) {
      // the run-time-radix body loops over a column's butterflies and
      // elements with any number of threads per column: fill the CTA up to
      // the thread cap (no idle warps in the persistent group's 256-thread
      // CTAs, more warps in the pass's own launch)
      const int tmax = dtype_cfg(sizeof(T) == 8).threads_max;
      const int tf = std::min(std::max(op.pp.Tf, tmax / std::max(op.pp.NB, 1)), op.pp.R);
      if (tf > op.pp.Tf) {
        op.pp.Tf = tf;
        op.pp.threads = op.pp.NB * tf;
        op.pp.ept = (op.pp.R + tf - 1) / tf;
      }
    }
    op.pp.smem_tw_elems = stage_inner_twiddles(op.pp, op.kfn != nullptr) ? op.pp.R : 0;
    if (sizeof(T) == 4 && (op.kfn || op.pp.tc == 1) && !P->plain_loads) pick_tma(op, P->dry);
    any_tma = any_tma || op.kfn_tma != nullptr;
    if (P->dry) continue;
    if (prepare_pass<T>(op.pp, op.dir, op.kfn) != cudaSuccess) return fail(FFTJ_ERR_CUDA, "cudaFuncSetAttribute failed");
  }
  if (any_tma && !P->dry) {
    if (cudaMalloc(&P->d_status, sizeof(unsigned)) != cudaSuccess ||
        cudaMemset(P->d_status, 0, sizeof(unsigned)) != cudaSuccess)
      return fail(FFTJ_ERR_CUDA, "status word allocation failed");
  }
  return FFTJ_OK;
}

int finish(fftj_plan_s* P, fftj_plan* out) {
  int frc = P->dtype == FFTJ_F32 ? finalize_passes<float>(P) : finalize_passes<double>(P);
  if (frc) return frc;
  wire(P->ops);
  int rc = alloc_workspace(P);
  if (rc) return rc;
  P->npasses = (int)P->ops.size();
  *out = P;
  g_err.clear();
  return FFTJ_OK;
}

}  // namespace

// Installs a planning call's schedule options on this host thread and
// restores the defaults when the call returns.
struct SchedScope {
  explicit SchedScope(const fftj_plan_opts_t* o) {
    g_sched = SchedOpts();
    if (!o) return;
    g_sched.tile = o->tile;
    g_sched.extra_passes = std::min(std::max(o->extra_passes, 0), 2);
    g_sched.order = std::max(o->order, 0);
    g_sched.tf_mult = std::min(std::max(o->tf_mult, 0), 4);
    g_sched.route = o->route;
    g_sched.threads_max = o->threads_max;
    g_sched.dry = o->dry != 0;
    g_sched.precision = (o->precision >= 0 && o->precision <= 2) ? o->precision : 0;
    g_sched.plain_loads = o->plain_loads != 0 ? 1 : 0;
    g_sched.f64_arith = o->f64_arith != 0 ? 1 : 0;
    g_sched.hvdh_factors = (o->hvdh_factors >= 0 && o->hvdh_factors <= 2) ? o->hvdh_factors : 0;
    g_sched.wide_axis = o->wide_axis == 1 ? 1 : 0;
  }
  ~SchedScope() { g_sched = SchedOpts(); }
};

extern "C" {

int fftj_plan_c2c(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch, int64_t idist,
                  int64_t odist, int dir, double scale) {
  return fftj_plan_c2c_ex(out, dtype, rank, dims, batch, idist, odist, dir, scale, nullptr);
}

int fftj_plan_c2c_ex(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch, int64_t idist,
                     int64_t odist, int dir, double scale, const fftj_plan_opts_t* opts) {
  if (!out) return fail(FFTJ_ERR_ARG, "null plan pointer");
  *out = nullptr;
  SchedScope scope(opts);
  std::vector<i64> d;
  if (int rc = check_dims(rank, dims, &d)) return rc;
  if (dtype != FFTJ_F32 && dtype != FFTJ_F64) return fail(FFTJ_ERR_ARG, "dtype must be F32 or F64");
  if (dir != -1 && dir != 1) return fail(FFTJ_ERR_ARG, "dir must be -1 or +1");
  if (batch < 1) return fail(FFTJ_ERR_ARG, "batch must be >= 1");
  std::unique_ptr<fftj_plan_s> P(new fftj_plan_s());
  P->dry = g_sched.dry;
  P->dtype = dtype;
  P->kind = 0;
  P->dims = d;
  P->n = 1;
  for (i64 v : d) P->n *= v;
  P->batch = batch;
  if (idist == 0) idist = P->n;
  if (odist == 0) odist = P->n;
  if (idist < P->n || odist < P->n) return fail(FFTJ_ERR_DIM, "idist/odist smaller than the transform");
  int rc = dtype == FFTJ_F32 ? plan_c2c_t<float>(P.get(), d, batch, idist, odist, dir, scale)
                             : plan_c2c_t<double>(P.get(), d, batch, idist, odist, dir, scale);
  if (rc) return rc;
  // a single pass over whole transforms (tile = full transforms) is in-place safe
  P->inplace_safe = P->ops.size() == 1 && P->ops[0].kind == OP_PASS && P->ops[0].pp.m == 1 &&
                    P->ops[0].pp.s == 1 && idist == odist;
  rc = finish(P.get(), out);
  if (rc) return rc;
  P.release();
  return FFTJ_OK;
}

int fftj_plan_r2c(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch, int64_t idist,
                  int64_t odist) {
  return fftj_plan_r2c_ex(out, dtype, rank, dims, batch, idist, odist, nullptr);
}

int fftj_plan_r2c_ex(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch, int64_t idist,
                     int64_t odist, const fftj_plan_opts_t* opts) {
  if (!out) return fail(FFTJ_ERR_ARG, "null plan pointer");
  *out = nullptr;
  SchedScope scope(opts);
  std::vector<i64> d;
  if (int rc = check_dims(rank, dims, &d)) return rc;
  if (dtype != FFTJ_F32 && dtype != FFTJ_F64) return fail(FFTJ_ERR_ARG, "dtype must be F32 or F64");
  if (batch < 1) return fail(FFTJ_ERR_ARG, "batch must be >= 1");
  std::unique_ptr<fftj_plan_s> P(new fftj_plan_s());
  P->dry = g_sched.dry;
  P->dtype = dtype;
  P->kind = 1;
  P->dims = d;
  P->n = 1;
  for (i64 v : d) P->n *= v;
  P->batch = batch;
  const i64 cn = P->n / d[0] * (d[0] / 2 + 1);
  if (idist == 0) idist = P->n;
  if (odist == 0) odist = cn;
  if (idist < P->n || odist < cn) return fail(FFTJ_ERR_DIM, "idist/odist smaller than the transform");
  int rc = dtype == FFTJ_F32 ? plan_r2c_t<float>(P.get(), d, batch, idist, odist)
                             : plan_r2c_t<double>(P.get(), d, batch, idist, odist);
  if (rc) return rc;
  rc = finish(P.get(), out);
  if (rc) return rc;
  P.release();
  return FFTJ_OK;
}

int fftj_plan_c2r(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch, int64_t idist,
                  int64_t odist, int normalized) {
  return fftj_plan_c2r_ex(out, dtype, rank, dims, batch, idist, odist, normalized, nullptr);
}

int fftj_plan_c2r_ex(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch, int64_t idist,
                     int64_t odist, int normalized, const fftj_plan_opts_t* opts) {
  if (!out) return fail(FFTJ_ERR_ARG, "null plan pointer");
  *out = nullptr;
  SchedScope scope(opts);
  std::vector<i64> d;
  if (int rc = check_dims(rank, dims, &d)) return rc;
  if (dtype != FFTJ_F32 && dtype != FFTJ_F64) return fail(FFTJ_ERR_ARG, "dtype must be F32 or F64");
  if (batch < 1) return fail(FFTJ_ERR_ARG, "batch must be >= 1");
  std::unique_ptr<fftj_plan_s> P(new fftj_plan_s());
  P->dry = g_sched.dry;
  P->dtype = dtype;
  P->kind = 2;
  P->dims = d;
  P->n = 1;
  for (i64 v : d) P->n *= v;
  P->batch = batch;
  const i64 cn = P->n / d[0] * (d[0] / 2 + 1);
  if (idist == 0) idist = cn;
  if (odist == 0) odist = P->n;
  if (idist < cn || odist < P->n) return fail(FFTJ_ERR_DIM, "idist/odist smaller than the transform");
  int rc = dtype == FFTJ_F32 ? plan_c2r_t<float>(P.get(), d, batch, idist, odist, normalized != 0)
                             : plan_c2r_t<double>(P.get(), d, batch, idist, odist, normalized != 0);
  if (rc) return rc;
  rc = finish(P.get(), out);
  if (rc) return rc;
  P.release();
  return FFTJ_OK;
}

// Launch op i of a plan (src/dst resolved from the plan's buffer ids).
static cudaError_t launch_op(fftj_plan_s* P, size_t i, void* const* bufs, bool via_ws, cudaStream_t st) {
  Op& op = P->ops[i];
  const void* src = bufs[op.src];
  void* dst = via_ws ? P->ws[0].p : bufs[op.dst];
  cudaError_t e = cudaSuccess;
  // the pipelined tensor-copy kernel where the pass has one and the source
  // is 16-byte aligned (a tensor map's base); its map is re-encoded when the
  // source address changes
  if (op.kind == OP_PASS && op.kfn_tma && P->d_status && ((uintptr_t)src & 15) == 0) {
    // single-pass tiles are 1-D bulk copies from `src` (no tensor map)
    if (op.tmap_src != src) op.tmap_src = (op.tma_mode == 0 || encode_tma(op, src)) ? src : nullptr;
    if (op.tmap_src == src) return tma_launch(op.kfn_tma, op.pp, op.tmap, src, dst, P->d_status, op.tma_grid, st);
  }
  if (P->dtype == FFTJ_F32) {
    switch (op.kind) {
      case OP_PASS: e = launch_pass<float>(op.pp, op.dir, op.kfn, src, dst, st); break;
      case OP_INTERP: e = launch_interp<float>(op.ip, src, dst, st); break;
      case OP_RPOST: e = launch_real_post<float>(op.rp, src, dst, st); break;
      case OP_COPY: e = launch_copy<float>(op.cp, src, dst, st); break;
      case OP_SOLVE: e = launch_solve<float>(op.sv, src, dst, st); break;
    }
  } else {
    switch (op.kind) {
      case OP_PASS: e = launch_pass<double>(op.pp, op.dir, op.kfn, src, dst, st); break;
      case OP_INTERP: e = launch_interp<double>(op.ip, src, dst, st); break;
      case OP_RPOST: e = launch_real_post<double>(op.rp, src, dst, st); break;
      case OP_COPY: e = launch_copy<double>(op.cp, src, dst, st); break;
      case OP_SOLVE: e = launch_solve<double>(op.sv, src, dst, st); break;
    }
  }
  return e;
}

int fftj_plan_c2c_from_tables(fftj_plan* out, int dtype, int64_t n, int64_t batch, int dir, double scale,
                              const double* omega, int64_t N, const fftj_resample_tables_t* rs) {
  if (!out) return fail(FFTJ_ERR_ARG, "null plan pointer");
  *out = nullptr;
  if (n < 1 || batch < 1) return fail(FFTJ_ERR_ARG, "transform length and batch must be positive");
  if (dir != -1 && dir != 1) return fail(FFTJ_ERR_ARG, "dir must be -1 or +1");
  if (!omega) return fail(FFTJ_ERR_ARG, "null root table");
  std::vector<int> primes;
  const bool smooth = smooth13(n, &primes);
  if (smooth) {
    if (rs) return fail(FFTJ_ERR_ARG, "resampling tables given for a 13-smooth length");
    if (N != n) return fail(FFTJ_ERR_DIM, "a 13-smooth length takes the roots of w_n (N = n)");
  } else {
    if (!rs || !rs->corr || !rs->wt || !rs->l0) return fail(FFTJ_ERR_ARG, "a non-smooth length needs resampling tables");
    std::vector<int> pm;
    if (rs->m < n || !smooth13(rs->m, &pm)) return fail(FFTJ_ERR_ARG, "the resampled grid m must be 13-smooth and >= n");
    if (N != rs->m) return fail(FFTJ_ERR_DIM, "a resampled length takes the roots of w_m (N = m)");
    if (rs->w < 1 || rs->w > 64) return fail(FFTJ_ERR_ARG, "interpolation taps must be 1..64");
    for (i64 k = 0; k < n; ++k)
      if (rs->l0[k] < -rs->m || rs->l0[k] >= rs->m) return fail(FFTJ_ERR_ARG, "l0 entries must lie in [-m, m)");
  }
  g_tables.omega = omega;
  g_tables.N = N;
  g_tables.rs = rs;
  // smooth lengths apply the scale in the last pass; resampled ones carry it in corr
  const int rc = fftj_plan_c2c_ex(out, dtype, 1, &n, batch, 0, 0, dir, smooth ? scale : 1.0, nullptr);
  g_tables = HostTables();
  return rc;
}

int fftj_execute(fftj_plan plan, const void* d_in, void* d_out, void* stream) {
  if (!plan) return fail(FFTJ_ERR_ARG, "null plan");
  if (!d_in || !d_out) return fail(FFTJ_ERR_ARG, "null data pointer");
  if (plan->dry) return fail(FFTJ_ERR_ARG, "a dry plan (opts.dry = 1) holds no tables and cannot execute");
  cudaStream_t st = (cudaStream_t)stream;
  fftj_plan_s* P = plan;
  void* bufs[4] = {const_cast<void*>(d_in), d_out, P->ws[0].p, P->ws[1].p};
  const bool via_ws = P->ops.size() == 1 && !P->inplace_safe && d_in == d_out;
  for (size_t i = 0; i < P->ops.size(); ++i) {
    const cudaError_t e = launch_op(P, i, bufs, via_ws, st);
    if (e != cudaSuccess) return fail(FFTJ_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
  }
  if (via_ws) {
    cudaError_t e = cudaMemcpyAsync(d_out, P->ws[0].p, P->ops[0].dst_bytes, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return fail(FFTJ_ERR_CUDA, std::string("copy failed: ") + cudaGetErrorString(e));
  }
  g_err.clear();
  return FFTJ_OK;
}

int fftj_plan_status(fftj_plan plan, void* stream) {
  if (!plan) return fail(FFTJ_ERR_ARG, "null plan");
  if (!plan->d_status) {
    g_err.clear();
    return FFTJ_OK;
  }
  if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return fail(FFTJ_ERR_CUDA, "execution failed");
  unsigned st = 0;
  if (cudaMemcpy(&st, plan->d_status, sizeof(st), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(FFTJ_ERR_CUDA, "status read failed");
  if (st) {
    cudaMemset(plan->d_status, 0, sizeof(unsigned));
    if (st & 2u)
      return fail(FFTJ_ERR_TIMEOUT,
                  "a pipelined pass gave up waiting for a tile's tensor copy and exited with copies in flight: "
                  "treat every result produced on this stream since the previous status check as lost");
    return fail(FFTJ_ERR_TIMEOUT, "a pipelined pass gave up waiting for a tile's tensor copy; its output is incomplete");
  }
  g_err.clear();
  return FFTJ_OK;
}

int fftj_plan_set_wait_limit(fftj_plan plan, uint64_t ns) {
  if (!plan) return fail(FFTJ_ERR_ARG, "null plan");
  if (ns < 1000) return fail(FFTJ_ERR_ARG, "wait limit below 1 us");
  for (auto& op : plan->ops) op.pp.tma_wait_ns = ns;
  g_err.clear();
  return FFTJ_OK;
}

int fftj_plan_debug_stall(fftj_plan plan, int extra_bytes) {
  if (!plan) return fail(FFTJ_ERR_ARG, "null plan");
  if (extra_bytes < 0 || extra_bytes > (1 << 20)) return fail(FFTJ_ERR_ARG, "extra bytes must be in [0, 2^20]");
  for (auto& op : plan->ops) op.pp.tma_extra_tx = extra_bytes;
  g_err.clear();
  return FFTJ_OK;
}

int fftj_profile_ops(fftj_plan plan, const void* d_in, void* d_out, void* stream, int reps, float* ms, int cap) {
  if (!plan || !d_in || !d_out || !ms || reps < 1) return fail(FFTJ_ERR_ARG, "null argument or reps < 1");
  if (plan->dry) return fail(FFTJ_ERR_ARG, "a dry plan cannot execute");
  if (d_in == d_out) return fail(FFTJ_ERR_ARG, "profiling needs distinct input and output buffers");
  fftj_plan_s* P = plan;
  const size_t k = P->ops.size();
  if ((size_t)cap < k) return fail(FFTJ_ERR_ARG, "cap smaller than the plan's op count");
  cudaStream_t st = (cudaStream_t)stream;
  void* bufs[4] = {const_cast<void*>(d_in), d_out, P->ws[0].p, P->ws[1].p};
  std::vector<cudaEvent_t> ev(k + 1);
  for (auto& e : ev) cudaEventCreate(&e);
  std::vector<double> acc(k, 0.0);
  int rc = FFTJ_OK;
  for (int r = 0; r < reps && rc == FFTJ_OK; ++r) {
    cudaEventRecord(ev[0], st);
    for (size_t i = 0; i < k && rc == FFTJ_OK; ++i) {
      if (launch_op(P, i, bufs, false, st) != cudaSuccess) rc = fail(FFTJ_ERR_CUDA, "kernel launch failed");
      cudaEventRecord(ev[i + 1], st);
    }
    if (rc == FFTJ_OK && cudaEventSynchronize(ev[k]) != cudaSuccess) rc = fail(FFTJ_ERR_CUDA, "execution failed");
    for (size_t i = 0; i < k && rc == FFTJ_OK; ++i) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
      acc[i] += t;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  for (size_t i = 0; i < k; ++i) ms[i] = (float)(acc[i] / reps);
  g_err.clear();
  return FFTJ_OK;
}

int fftj_plan_get_info(fftj_plan plan, fftj_plan_info_t* info) {
  if (!plan || !info) return fail(FFTJ_ERR_ARG, "null argument");
  std::memset(info, 0, sizeof(*info));
  info->route = plan->route;
  info->npasses = (int)plan->ops.size();
  info->n = plan->n;
  info->batch = plan->batch;
  info->resample_m = plan->resample_m;
  info->resample_w = plan->resample_w;
  for (size_t i = 0; i < plan->pass_R.size() && i < 8; ++i) info->pass_radix[i] = plan->pass_R[i];
  info->workspace_bytes = plan->ws[0].bytes + plan->ws[1].bytes;
  info->table_bytes = plan->table_bytes;
  info->nops = (int)plan->ops.size();
  info->dry = plan->dry ? 1 : 0;
  for (const auto& op : plan->ops) info->tma_passes += op.kfn_tma != nullptr ? 1 : 0;
  // FNV-1a over everything that shapes the launches
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](int64_t v) {
    for (int i = 0; i < 8; ++i) {
      h ^= (uint64_t)((v >> (8 * i)) & 0xff);
      h *= 1099511628211ull;
    }
  };
  mix(plan->route);
  mix(plan->kind);
  mix(plan->dtype);
  int pi = 0;
  for (auto& op : plan->ops) {
    mix(op.kind);
    if (op.kind == OP_PASS) {
      const PassParams& pp = op.pp;
      if (op.kfn) info->specialized_passes++;
      info->fx_passes += pp.fx ? 1 : 0;
      if (pp.tc) {
        // the pipelined precision-form kernel runs its first sub-stage on
        // the tensor cores; the run-time kernel every radix-16 sub-stage
        // that fits
        if (op.kfn_tma) {
          info->tc_substages += 1;
        } else {
          for (int i = 0; i < pp.nsub; ++i) info->tc_substages += tc16_substage_fits(pp, i) ? 1 : 0;
        }
      }
      if (pi < 8) {
        info->pass_tile[pi] = pp.NB * pp.R;
        info->pass_threads[pi] = pp.threads;
        info->pass_ctas[pi] = (int64_t)pp.tiles_q * pp.tiles_p * pp.tiles_b;
      }
      pi++;
      for (int64_t v : {(int64_t)pp.R, (int64_t)pp.P, (int64_t)pp.Q, (int64_t)pp.NBt, (int64_t)pp.Tf,
                        (int64_t)pp.threads, (int64_t)pp.nsub, (int64_t)pp.tw_mode, (int64_t)pp.load_op, (int64_t)pp.tc,
                        (int64_t)pp.fx,
                        (int64_t)(uintptr_t)op.kfn, (int64_t)(uintptr_t)op.kfn_tma})
        mix(v);
      for (int i = 0; i < pp.nsub; ++i) mix(pp.sub[i].r);
    } else if (op.kind == OP_INTERP) {
      mix(op.ip.w);
      mix(op.ip.m);
    } else if (op.kind == OP_SOLVE) {
      mix(op.sv.L);
      mix(op.sv.H);
      mix(op.sv.B);
    } else if (op.kind == OP_COPY) {
      mix(op.cp.mode);
    }
  }
  info->schedule_hash = h;
  return FFTJ_OK;
}

int fftj_plan_features(fftj_plan plan, float* out, int cap) {
  if (!plan || !out || cap < FFTJ_NFEATURES) return fail(FFTJ_ERR_ARG, "null plan/output or cap < FFTJ_NFEATURES");
  auto lg = [](double x) { return x > 0 ? std::log2(x) : 0.0; };
  double f[FFTJ_NFEATURES] = {0};
  const bool f64 = plan->dtype == FFTJ_F64;
  f[0] = lg((double)plan->n);
  f[1] = lg((double)plan->batch);
  f[2] = f64 ? 1 : 0;
  f[3] = plan->kind == 1;
  f[4] = plan->kind == 2;
  f[5] = plan->route == FFTJ_ROUTE_RESAMPLE;
  f[6] = plan->route == FFTJ_ROUTE_HVDH;
  f[7] = plan->route == FFTJ_ROUTE_ND;
  f[8] = (double)plan->ops.size();
  int np = 0, spec = 0;
  double bytes = 0, ctas = 0;
  for (auto& op : plan->ops) {
    bytes += 2.0 * (double)op.dst_bytes;
    if (op.kind == OP_PASS) {
      const PassParams& pp = op.pp;
      const double c = (double)pp.tiles_q * pp.tiles_p * pp.tiles_b;
      ctas += c;
      if (np < 3) {
        f[10 + np] = lg(pp.R);
        f[13 + np] = lg((double)pp.NB * pp.R);
        f[16 + np] = lg(pp.threads);
        f[19 + np] = lg(c);
      }
      np++;
      if (op.kfn) spec++;
    } else {
      double total = 0;
      if (op.kind == OP_INTERP) total = (double)op.ip.n * op.ip.nbatch * std::max<int64_t>(op.ip.inner, 1);
      else if (op.kind == OP_RPOST) total = (double)(op.rp.h / 2 + 1) * op.rp.nbatch;
      else if (op.kind == OP_COPY) total = (double)op.cp.n * op.cp.nbatch;
      else if (op.kind == OP_SOLVE) total = (double)op.sv.nbatch * op.sv.nchunk;
      ctas += std::ceil(total / 256.0);
    }
  }
  f[9] = np;
  f[22] = np ? (double)spec / np : 0;
  f[23] = lg(bytes);
  const double grid = (double)(plan->resample_m ? plan->resample_m : plan->n);
  f[24] = lg(grid);
  i64 g = plan->resample_m ? plan->resample_m : plan->n;
  while (g > 1 && g % 2 == 0) g /= 2;
  f[25] = lg((double)g);
  f[26] = np - spec;
  f[27] = lg(ctas);
  for (int i = 0; i < FFTJ_NFEATURES; ++i) out[i] = (float)f[i];
  return FFTJ_OK;
}

int fftj_plan_workspace_bytes(fftj_plan plan, size_t* bytes) {
  if (!plan || !bytes) return fail(FFTJ_ERR_ARG, "null argument");
  *bytes = plan->ws[0].bytes + plan->ws[1].bytes;
  return FFTJ_OK;
}

int fftj_plan_destroy(fftj_plan plan) {
  delete plan;
  return FFTJ_OK;
}

const char* fftj_last_error_string(void) { return g_err.c_str(); }

const char* fftj_version(void) { return "fftj-gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
