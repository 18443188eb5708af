// TEST INFRASTRUCTURE ONLY — never linked into, loaded by, or called from the
// product library. Used by tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg as the checker and the timed CPU reference.
//
// CPU restatement of FFTJ.jl's transform path (reference: oscardssmith/FFTJ.jl,
// pure Julia). Julia is not available on either machine, so this C++ code
// restates the reference's algorithms (factorization, radix tower, stage index
// maps, butterflies, four-step, resampling, real and N-d plans, routing) and
// serves as "the FFTJ CPU plan" for parity and for the threaded CPU baseline.
// Parity unpinned: the reference's tests hold no stored vectors and no
// outputs of the reference itself could be produced here (no Julia
// toolchain), so the restatement is checked against an FP64 direct DFT with
// double-double accumulation and against numpy's pocketfft at the
// reference's own test sizes and tolerance classes (test/runtests.jl).
#pragma once
#include <cstdint>

extern "C" {

// Route of a 1-D plan (FFTJ plan types, src/plan.jl:192-206).
enum orc_route {
  ORC_FFTPLAN = 0,    // direct Stockham chain (src/plan.jl:48-58)
  ORC_FOURSTEP = 1,   // four-step (src/fourstep.jl:130-156)
  ORC_RESAMPLE = 2,   // oversampled resampling (src/resample.jl:175-182)
  ORC_HVDH = 3,       // Gaussian resampling (src/hvdh.jl:30-58)
  ORC_COMPOSITE = 5,  // smooth part first, then batched resampling (src/composite.jl:10-101)
  ORC_SPLIT = 6,      // decimation in time into HvdH sub-transforms (src/composite.jl:103-280)
  ORC_NDPLAN = 4,     // N-d plan, one pass per dimension (src/ndplan.jl:57-118)
  ORC_FS2 = 7,        // 2-D N-d plan run as Fs2Plan: strided dim 2 first, then the rows (src/fourstep.jl:500-552)
};

// Host SIMD width FFTJ would see (src/kernels.jl:11-22). 128 = NEON (the GPU
// box's Grace host), 512 = AVX-512. Affects routing and tower shapes only.
void orc_set_vector_bits(int bits);
int orc_get_vector_bits(void);

// 1-D complex plan. dtype 0 = F32, 1 = F64. D = -1 forward, +1 inverse.
// scale_mode: 0 = FFTJ default (1 forward, 1/n inverse), 1 = unnormalized.
void* orc_plan_c2c(int dtype, int64_t n, int D, int scale_mode, int nthreads);
int orc_plan_route(void* plan);
int64_t orc_plan_info(void* plan, int64_t* out, int64_t cap);
// x, y: interleaved complex (T pairs), batch transforms at stride n.
// Batches run one after another, threads inside each transform (as FFTJ).
int orc_execute_c2c(void* plan, const void* x, void* y, int64_t batch);
void orc_destroy(void* plan);

// Real transforms (src/real.jl). rfft: n reals -> n/2+1 complex.
// irfft (normalized=1) / brfft (normalized=0): n/2+1 complex -> n reals.
void* orc_plan_rfft(int dtype, int64_t n, int nthreads);
void* orc_plan_irfft(int dtype, int64_t n, int normalized, int nthreads);
int orc_execute_rfft(void* plan, const void* x, void* y, int64_t batch);
int orc_execute_irfft(void* plan, const void* x, void* y, int64_t batch);

// N-d complex plans (src/ndplan.jl), column-major dims (dim 1 fastest).
// kind: 0 fft, 1 ifft (1/len), 2 bfft.
void* orc_plan_nd(int dtype, int rank, const int64_t* dims, int kind, int nthreads);
int orc_execute_nd(void* plan, const void* x, void* y);
// N-d real: rfft (dims = real dims) and irfft/brfft (dims = real dims).
void* orc_plan_rfft_nd(int dtype, int rank, const int64_t* dims, int nthreads);
void* orc_plan_irfft_nd(int dtype, int rank, const int64_t* dims, int normalized, int nthreads);
// 1 when the plan's dim-1 edge runs batched (pencils as lanes): the complex
// dim-1 chain without the small-stride layout, or the batched real edge.
int orc_plan_nd_batched(void* plan);
// FFTJ's polynomial exp (_vexp) that seeds the HvdH recurrences, in F32
// (dtype 0, x rounded to F32 first) or F64.
double orc_vexp(int dtype, double x);
int orc_execute_rfft_nd(void* plan, const void* x, void* y);
int orc_execute_irfft_nd(void* plan, const void* x, void* y);

// Plans of a given type, built directly as the reference's tests build them
// (FFTJ._hvdh, FFTJ._composite, FFTJ._split). factors: 0 :auto, 1 :table
// (factors tabulated at plan time), 2 :fly (rebuilt every call). NULL when
// the reference throws ArgumentError (orc_last_error gives the message).
void* orc_plan_hvdh(int dtype, int64_t n, int D, int scale_mode, int factors);
void* orc_plan_composite(int dtype, int64_t n, int D, int scale_mode);
void* orc_plan_split(int dtype, int64_t n, int D, int scale_mode);
const char* orc_last_error(void);

// FP64 direct DFT, exact integer angle reduction, double-double accumulation.
// sign = -1 forward (no scaling), +1 backward (no scaling).
void orc_dft_f64(int64_t n, const double* x, double* y, int sign);

// Thread pool used by the threaded plans (src/threads.jl:15-41 restated).
int orc_max_threads(void);

// Accessors used to cross-check the product planner's tables.
int orc_factor_radices(int64_t n, int64_t* a, int64_t* primes, int64_t* counts, int64_t cap);
int64_t orc_nextsmooth(int64_t n);
int64_t orc_nextsmooth7(int64_t n);
// resampling parameters for (dtype, n): returns m, fills w and beta.
int64_t orc_resample_params(int dtype, int64_t n, int64_t* w, double* beta);
}
