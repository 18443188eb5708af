/*
 * fftj.h — C ABI of the GB300-native (sm_103a) FFTJ transform library.
 *
 * Drop-in boundary for FFTJ.jl's plan surface (oscardssmith/FFTJ.jl). FFTJ's
 * boundary is Julia functions, not an FFI; each entry point below names the
 * reference function it replaces so that a Julia front end (api.jl style)
 * can ccall it with device pointers. Plain C types only.
 *
 * Conventions carried over from the reference:
 *  - Layout: interleaved complex (re, im) of float or double, column-major
 *    dims (dim 1 fastest); rfft output has n1/2+1 rows along dim 1.
 *  - Scaling: forward 1, ifft 1/n, bfft 1 (src/plan.jl:97); irfft 1/n,
 *    brfft 1 (src/real.jl:54-73).
 *  - Errors: FFTJ throws ArgumentError (bad length, region, kwargs) and
 *    DimensionMismatch (wrong lengths) (src/plan.jl:171, 361-362;
 *    src/api.jl:103-105). Here they are FFTJ_ERR_ARG / FFTJ_ERR_DIM status
 *    codes with a message in fftj_last_error_string().
 *  - A plan owns its device tables and workspace; one plan runs on one stream
 *    at a time (FFTJ plans own scratch and are not reentrant,
 *    src/plan.jl:52-55). Execution never allocates and never synchronises
 *    the host (FFTJ's "@allocated == 0" contract, test/runtests.jl:33).
 *  - in == out is allowed (FFTJ's in-place plans wrap out-of-place ones,
 *    src/api.jl:11-24).
 */
#ifndef FFTJ_H
#define FFTJ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fftj_plan_s* fftj_plan;

typedef enum {
  FFTJ_OK = 0,
  FFTJ_ERR_ARG = 1,         /* ArgumentError */
  FFTJ_ERR_DIM = 2,         /* DimensionMismatch */
  FFTJ_ERR_CUDA = 3,        /* CUDA runtime failure */
  FFTJ_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
  FFTJ_ERR_UNSUPPORTED = 5  /* valid request this build does not implement */
} fftj_status;

typedef enum { FFTJ_F32 = 0, FFTJ_F64 = 1 } fftj_dtype;

/* Algorithm chosen by the planner (FFTJ plan types, src/plan.jl:192-206). */
typedef enum {
  FFTJ_ROUTE_DIRECT = 0,    /* FFTPlan: smooth length, Stockham passes */
  FFTJ_ROUTE_FOURSTEP = 1,  /* FourStepPlan: multi-pass out-of-cache length */
  FFTJ_ROUTE_RESAMPLE = 2,  /* ResamplePlan: non-smooth length */
  FFTJ_ROUTE_HVDH = 3,      /* HvdhPlan */
  FFTJ_ROUTE_ND = 4         /* NdPlan / RfftNdPlan / IrfftNdPlan */
} fftj_route;

typedef struct {
  int route;            /* fftj_route */
  int npasses;          /* HBM passes (kernel launches over the data) */
  int64_t n;            /* transform length (product of dims) */
  int64_t batch;
  int64_t resample_m;   /* resampled grid length (0 unless RESAMPLE) */
  int64_t resample_w;   /* interpolation taps */
  int pass_radix[8];    /* points per butterfly of each pass */
  size_t workspace_bytes;
  size_t table_bytes;
  int specialized_passes; /* passes run by compile-time specialised kernels */
} fftj_plan_info_t;

/*
 * 1-D / N-d complex plan.
 * Replaces plan_fft / plan_ifft / plan_bfft (src/plan.jl:207-213) and the
 * array-based N-d planners (src/api.jl:107-154, src/ndplan.jl:57-118).
 *   dims[rank]: column-major lengths (rank 1 = 1-D).
 *   batch, idist, odist: transforms at element strides idist/odist (complex
 *     elements); 0 means dense (prod(dims)). Batch is an extension: FFTJ
 *     plans one array and callers loop.
 *   dir: -1 forward, +1 backward. scale: multiplies the result
 *     (1 for fft/bfft, 1/n for ifft).
 */
int fftj_plan_c2c(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch,
                  int64_t idist, int64_t odist, int dir, double scale);

/*
 * Real-input forward plan: prod(dims) reals -> (dims[0]/2+1)*prod(dims[1:])
 * complex. Replaces plan_rfft(T, n) (src/real.jl:41-52) and the N-d rfft
 * planner (src/api.jl:347-352, src/ndplan.jl:369-390). idist/odist in reals /
 * complex elements (0 = dense).
 */
int fftj_plan_r2c(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch,
                  int64_t idist, int64_t odist);

/*
 * Complex-to-real backward plan, dims = the REAL output dims. normalized=1
 * gives irfft (1/n), 0 gives brfft. Replaces plan_irfft / plan_brfft
 * (src/real.jl:57-73, src/api.jl:353-370, src/ndplan.jl:455-481).
 */
int fftj_plan_c2r(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch,
                  int64_t idist, int64_t odist, int normalized);

/*
 * Apply a plan: FFTJ's p(y, x) / mul!(y, p, x) / p * x (src/api.jl:34-55,
 * src/plan.jl:359-396). d_in, d_out: device pointers; stream: a
 * cudaStream_t (NULL = legacy default stream). Asynchronous; no allocation.
 */
int fftj_execute(fftj_plan plan, const void* d_in, void* d_out, void* stream);

/* Size and algorithm of a plan (FFTJ: size(p) and the plan type). */
int fftj_plan_get_info(fftj_plan plan, fftj_plan_info_t* info);

/* Device workspace owned by the plan, in bytes. */
int fftj_plan_workspace_bytes(fftj_plan plan, size_t* bytes);

/* Free the plan's device tables and workspace. NULL is a no-op. */
int fftj_plan_destroy(fftj_plan plan);

/* Message for the last error on this host thread ("" after success). */
const char* fftj_last_error_string(void);

/* Library version string. */
const char* fftj_version(void);

/*
 * Allocation-free complex transform. No counterpart in the reference: it is
 * for callers that cannot allocate device memory when they transform, such
 * as code recording a CUDA stream capture (cudaMalloc cannot be captured),
 * real-time loops that forbid allocation after start-up, and hosts that own
 * all device memory through their own pool. It creates no plan and calls no
 * cudaMalloc, cudaFree or other allocating routine: its scratch is a
 * file-scope static device array of 64 MiB (1 MiB of twiddle tables,
 * regenerated on the device on every call, and 63 MiB for the intermediate
 * of a two-pass transform) that every GPU loading the library holds until
 * exit. Limits: n 13-smooth and done in one or two passes (n <= 2^20), and
 * for two passes batch * n * sizeof(complex) <= 63 MiB; larger requests
 * return FFTJ_ERR_ARG / FFTJ_ERR_UNSUPPORTED with a message. d_in/d_out hold
 * batch dense transforms; in == out is allowed. The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) and should
 * come before any stream capture. All calls share the one array: calls that
 * overlap on the GPU (other streams, other threads) race and must be
 * serialised by the caller. Nothing in the array needs to start at zero.
 */
int fftj_execute_noalloc_c2c(int dtype, int64_t n, int64_t batch, int dir, double scale, const void* d_in,
                             void* d_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FFTJ_H */
