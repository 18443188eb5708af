// Internal structures shared by the host planner (planner.cpp) and the
// sm_103a kernels (kernels.cu).
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace fftj {

// q = n / d for 0 <= n < 2^31 by multiply-high and shift (d = 1: q = n).
struct FastDiv {
  uint32_t d = 1, mul = 0, shr = 0;
  FastDiv() {}
  explicit FastDiv(uint32_t div) : d(div) {
    if (div <= 1) { d = 1; mul = 0; shr = 0; return; }
    uint32_t l = 0;
    while ((1ull << l) < div) ++l;  // ceil(log2 d)
    uint32_t p = 31 + l;
    unsigned long long m = ((1ull << p) + div - 1) / div;  // ceil(2^p / d)
    mul = (uint32_t)m;
    shr = p - 32;
  }
#ifdef __CUDACC__
  __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
    return d == 1 ? n : (__umulhi(n, mul) >> shr);
#else
    return n / d;
#endif
  }
#endif
};

constexpr int kMaxSub = 12;

// One radix sub-stage inside a pass: Stockham stage of radix r on the
// pass's R-point sub-transforms at current length L = R / S.
struct SubStage {
  int r;
  int S;         // stride R / L (product of the earlier sub-radices)
  FastDiv fS;    // divide by S
  int Rr;        // R / r
};

enum LoadOp : int {
  LOAD_PLAIN = 0,     // complex x[b*idist + g]
  LOAD_DECONV = 1,    // resampling: deconvolve and zero-pad n -> m
  LOAD_C2R_PRE = 2,   // irfft even pre-pass Z[k] from X[k], conj X[h-k]
  LOAD_REAL = 3,      // real x -> (x, 0)
  LOAD_SPREAD = 4,    // HvdH: Gaussian spread of the input onto the t-grid
};

// Parameters of one Stockham super-radix pass over the data: radix-R
// butterflies (R points each, an R-point DFT done in shared memory),
// reading x[s*p + j*m*s + q] and writing y[R*s*p + j*s + q] * w_ncur^(p*j).
struct PassParams {
  int R;
  int nsub;
  SubStage sub[kMaxSub];
  // tile: NBt batches x P butterflies p x Q lanes q, NB = NBt*P*Q columns
  int P, Q, NBt, NB;
  FastDiv fQ, fP, fR, fNB;
  int64_t m, s, ncur;
  int64_t in_bstride, out_bstride, nbatch;
  uint32_t tiles_q, tiles_p, tiles_b;
  FastDiv ftq, ftp;
  // outer twiddle: 0 none, 1 full table tw[p*R + j], 2 two-level hi/lo
  int tw_mode;
  int tw_shift;            // K = 1 << tw_shift for two-level
  const void* tw_full;
  const void* tw_hi;
  const void* tw_lo;
  const void* twR;         // w_R^t, t < R (inner twiddles, sign of the pass)
  double scale;            // applied on store when != 1
  int smem_elems;          // padded elements per buffer
  int smem_tw_elems;       // extra shared elements (recipe kernels stage w_R^t there)
  int tc;                  // radix-16 sub-stages on tensor cores: 0 off, 1 FP16 hi+lo, 2 BF16 hi+lo (F32)
  int fx;                  // 1: ComplexF64 data computed in block fixed point (fx64.cuh), twiddles Q61
  int fx_cols;             // ints of shared memory for the column exponents (fx: NB, else 0)
  int fx_b0;               // fx: headroom bits of the inputs (61 - ceil(log2 r0))
  int fx_sht;              // fx: sum of the sub-stage boundary shifts (ceil(log2 r) of radices 2..)
  int threads;
  int Tf;                  // threads per tile column (threads = NB * Tf)
  int ept;                 // elements per thread per column (ceil(R / Tf))
  int load_rows;           // 1: lanes walk j (contiguous input rows), 0: lanes walk columns
  int store_rows;          // 1: lanes walk j (contiguous output rows), 0: lanes walk columns
  // fused load op parameters
  int load_op;
  int64_t ld_n, ld_m, ld_hp;     // DECONV: n, m, ceil(n/2); C2R_PRE: h = ld_n
  int64_t ld_stride;             // input batch stride of the raw input
  int64_t ld_inner;              // DECONV along a strided axis: inner stride (1 = contiguous)
  const void* ld_tab;            // DECONV: corr[n]; C2R_PRE: w[h], or hi[h >> ld_sh] when ld_sh > 0
  const void* ld_tab2;           // C2R_PRE two-level: lo[2^ld_sh]
  const void* ld_tab3;           // C2R_PRE first pass of several: w_n^(m t) = w_2R^t, t < R (or nullptr)
  int ld_sh;                     // C2R_PRE: 0 one table, else the two-level split
  double ld_pre;                 // C2R_PRE pair factor (1/2 or 1)
  int ld_w;                      // SPREAD: taps per grid row
  const int32_t* ld_l0;          // SPREAD: first input row of each grid row
  // pipelined tensor-copy kernel (pass_tma.cuh)
  int tma_rows;                  // tile rows per box copy (a divisor of R, <= 256)
  int tma_buf;                   // elements per tile buffer (a multiple of 16)
  int tma_extra_tx;              // test hook: bytes a tile's barrier expects beyond its copies (0)
  uint64_t tma_wait_ns;          // bound of each wait for a tile's copies
};

// HvdH banded solve: thread per (batch, chunk of L rows + 2H halo rows).
struct SolveParams {
  int64_t n, t, L, H, R, nchunk, nbatch;
  int64_t g_bstride, y_bstride;
  int64_t inner;             // lanes of a strided axis (HvPass; row r of lane i at r*inner + i), 0/1: none;
                             //   nbatch = outer blocks x inner, the strides are per outer block
  int B;
  double sc;                 // scale * n / t
  const void* lf;            // nchunk*R*B multipliers
  const void* uf;            // nchunk*R*(B+1): 1/U_ii, U_{i,i+1..i+B}
  const int32_t* oi;         // nchunk*R output index (-1: identity row)
  void* zw;                  // R * nbatch * nchunk forward-substitution scratch
  const void* tw;            // split route: w_(tw_s * n)^(r * o) applied to output o of sub-transform b,
  int64_t tw_s;              //   r = b mod tw_s (nullptr: none)
  // factors rebuilt in the solve (FFTJ factors = :fly) instead of read from
  // lf/uf/oi: per chunk the column state e = 2 t l' - 2 n q + n at its first
  // column (q = q0 - B) and the output index Delta l' mod n of its first row
  int fly;
  double a;                  // Gaussian exponent a = pi alpha^2
  int64_t delta;             // t - n
  const int64_t* se;         // nchunk: column state at column -B
  const int64_t* so;         // nchunk: output index of the first unknown at or after row 0
  void* uw;                  // R * (B + 1) * nbatch * nchunk: U rows of each thread's chunk
  int32_t* ow;               // R * nbatch * nchunk: output index of each row (-1: identity row)
};

// Resampling interpolation: y[b*ody + k] = sum_i wt[k*w+i] g[b*m + (l0[k]+i) mod m]
struct InterpParams {
  int64_t n, m, w, nbatch;
  int64_t g_bstride, y_bstride;
  int64_t inner;  // inner stride of the transformed axis (1 = contiguous)
  const void* wt;
  const int32_t* l0;
};

// rfft even post-pass: Y[k] (k = 0..h) from Z (length h) per batch.
struct RealPostParams {
  int64_t h, nbatch, z_bstride, y_bstride;
  const void* tw;   // e^{-2 pi i k/n}, k = 0..h/2; or hi[k >> sh] when sh > 0
  const void* tw2;  // two-level: lo[2^sh]
  int sh;           // 0: one table, else w^k = hi[k >> sh] lo[k & (2^sh - 1)]
};

// Generic elementwise helpers for odd-length real transforms.
struct CopyParams {
  int64_t n, nbatch, in_bstride, out_bstride;
  // 0: real -> complex, 1: hermitian expand (n real), 2: complex -> real,
  // 3: complex copy of n entries, 4: irfft pre-pass Z[k], k < n = h,
  // 5: decimation, row r of the output = x[r + s j], j < n / s (s = nc)
  // 6: twiddled transpose, output k2 + s j1 = x[j1 + p k2] w_n^(j1 k2) (s = nc)
  int mode;
  int64_t nc;          // complex length per batch (mode 1); s (modes 5, 6)
  const void* tab;     // mode 4: e^{+2 pi i k / 2h}; mode 6: w_n^e, e < n
  double pre;          // mode 4: pair factor (1/2 irfft, 1 brfft)
};

// Block fixed-point compute type of the ComplexF64 passes (fx64.cuh).
struct Fx;

// A pass kernel specialised at compile time for one radix sequence.
struct RecipeEntry {
  int f64, dir, load_op;
  int mode;      // 0 row load + row store, 1 fused load + row store, 2 fused both
  int radix[6];  // zero-terminated
  int Tf;        // threads per tile column the kernel was built for
  int nb;        // tile columns the kernel was built for (0: any)
  const void* fn;
  int tc = 0;    // precision form of the kernel (1: FP16 hi + lo tensor-core first sub-stage), 0 plain
};
template <typename T, int DIR>
const RecipeEntry* recipe_table(int* count);
// Pipelined tensor-copy pass kernels (F32, LOAD_PLAIN, modes 0, 1 and 2; nb
// = the exact tile column count). Signature:
// (PassParams, CUtensorMap, const float2* in, float2* out, unsigned* status).
const RecipeEntry* tma_table(int dir, int* count);
// Their precision-form variants (tc = 1), same signature.
const RecipeEntry* tma_tc_table(int* count);
size_t tma_smem_bytes(const PassParams& pp);
int tma_prepare(const void* fn, const PassParams& pp);
cudaError_t tma_launch(const void* fn, const PassParams& pp, const CUtensorMap& map, const void* in, void* out,
                       unsigned* status, int grid, cudaStream_t st);

// fn: a recipe kernel (RecipeEntry::fn) or nullptr for the generic kernel.
// Planner pieces shared by the plan builder and the allocation-free entry
// point (all heap-free).
struct DtypeCfg {
  int esize;        // bytes per complex element
  int tile_max;     // preferred elements per CTA tile (one shared buffer)
  int tile_cap;     // largest tile (shared memory / 16 elements per thread)
  int threads_max;  // CTA size bound of the kernel
  int rmax_multi;   // largest per-pass radix when more than one pass
  int min_run;      // minimum contiguous elements per tile row (coalescing)
};
// Schedule options of the plan being built on this host thread (set by the
// fftj_plan_*_ex entry points for the duration of one planning call; all
// zero otherwise, which is the default schedule).
struct SchedOpts {
  int tile = 0;
  int extra_passes = 0;
  int order = 0;
  int tf_mult = 0;
  int route = 0;
  int threads_max = 0;
  int precision = 0;
  int plain_loads = 0;
  int f64_arith = 0;
  int hvdh_factors = 0;
  int wide_axis = 0;
  bool dry = false;
};
extern thread_local SchedOpts g_sched;

DtypeCfg dtype_cfg(bool f64);
int pass_radices(int64_t n, bool f64, bool strided, int64_t* Rs, int cap);
int sub_radices(int64_t R, int* out, int cap);
int pass_geometry(PassParams& pp, bool f64, int64_t R, int64_t m, int64_t s, int64_t ncur, int64_t nbatch,
                  int64_t ibs, int64_t obs, bool wide = false);
// the one-pass strided F32 axis: its length and tile columns
constexpr int64_t kWideR = 4096;
constexpr int kWideCols = 4;
void outer_twiddle_layout(PassParams& pp, bool f64);
const void* pick_pass_kernel(bool f64, int dir, const PassParams& pp);
bool stage_inner_twiddles(const PassParams& pp, bool recipe);
bool tc16_substage_fits(const PassParams& pp, int i);
bool has_tc16_substage(const PassParams& pp);
void set_error(const char* msg);

template <typename T>
cudaError_t launch_pass(const PassParams& pp, int dir, const void* fn, const void* in, void* out,
                        cudaStream_t st);
template <typename T>
cudaError_t launch_interp(const InterpParams& ip, const void* g, void* y, cudaStream_t st);
template <typename T>
cudaError_t launch_real_post(const RealPostParams& rp, const void* z, void* y, cudaStream_t st);
template <typename T>
cudaError_t launch_copy(const CopyParams& cp, const void* in, void* out, cudaStream_t st);
template <typename T>
cudaError_t launch_solve(const SolveParams& sp, const void* g, void* y, cudaStream_t st);
// Opt a pass configuration into the dynamic shared memory it needs.
template <typename T>
cudaError_t prepare_pass(const PassParams& pp, int dir, const void* fn);

}  // namespace fftj
