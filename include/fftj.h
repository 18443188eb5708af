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
  FFTJ_ROUTE_ND = 4,        /* NdPlan / RfftNdPlan / IrfftNdPlan */
  FFTJ_ROUTE_SPLIT = 5,     /* SplitPlan: n = s p, s 7-smooth, decimation in time, p by Gaussian resampling */
  FFTJ_ROUTE_COMPOSITE = 6  /* CompositePlan: n = p s, decimation in frequency, p along s lanes by HvPass / RsPass */
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
  uint64_t schedule_hash; /* identifies the launch schedule (equal hash: same kernels, tiles, threads) */
  int pass_tile[8];       /* elements per CTA tile of each pass */
  int pass_threads[8];    /* threads per CTA of each pass */
  int64_t pass_ctas[8];   /* CTAs (tiles) of each pass */
  int nops;               /* kernel launches per execution (passes + elementwise ops) */
  int dry;                /* 1: planned without tables or workspace (cannot execute) */
  int tc_substages;       /* radix-16 sub-stages run on tensor cores (opts.precision != 0) */
  int tma_passes;         /* passes with a pipelined tensor-copy kernel (used when the input is 16-byte aligned) */
  int fx_passes;          /* ComplexF64 passes computed in block fixed point (integer pipes) */
} fftj_plan_info_t;

/*
 * Schedule options. No counterpart in the reference's API: FFTJ fixes its
 * schedule from the vector width and cache thresholds (src/plan.jl:105-151,
 * src/fourstep.jl:166-230); here the same choices -- radix split and order,
 * tile shape, threads per transform, route for non-smooth lengths -- are
 * exposed so that an autotuner can search them. All-zero = the planner's
 * default schedule. Options that cannot apply to a length are ignored.
 */
typedef struct {
  int32_t tile;          /* max elements per CTA tile (256 .. 8192 F32 / 4096 F64); 0 = default */
  int32_t extra_passes;  /* HBM passes beyond the fewest that fit (0, 1, 2) */
  int32_t order;         /* k-th lexicographic permutation of the pass radices (0 = largest first) */
  int32_t tf_mult;       /* threads per transform column = the minimum x tf_mult (0/1 = minimum) */
  int32_t route;         /* non-smooth lengths: 0 planner, 1 resampling, 2 Gaussian (HvdH; even lengths
                            by the split route), 4 CompositePlan (any 7-smooth part >= 2); any length:
                            3 Gaussian resampling at full length, as FFTJ._hvdh (FFTJ_ERR_ARG when no
                            smooth t is coprime to n) */
  int32_t threads_max;   /* cap on threads per CTA (0 = 512 F32 / 256 F64) */
  int32_t dry;           /* 1: plan the schedule only (no tables, no workspace, cannot execute) */
  int32_t precision;     /* F32 radix-16 sub-stages: 0 FP32 butterflies, 1 FP16 hi+lo tensor-core GEMM,
                            2 BF16 hi+lo tensor-core GEMM (FP32 accumulation, FP32 twiddles) */
  int32_t plain_loads;   /* 1: one-tile-per-CTA kernels only (no pipelined tensor-copy passes) */
  int32_t f64_arith;     /* ComplexF64 passes: 0 block fixed point on the integer pipes (default), 1 FP64
                            butterflies on the FP64 pipe (run-time-radix kernel) */
  int32_t hvdh_factors;  /* Gaussian resampling's banded-solve factors (FFTJ factors=): 0 auto (tables up to
                            1 GiB, else rebuilt per call), 1 tables, 2 rebuilt per call (:fly) */
  int32_t wide_axis;     /* 1: a strided F32 axis of length 4096 (inner extent a multiple of 4) runs as one
                            pass of 4-column tiles, so 4096 x 4096 sweeps HBM twice as FFTJ's Fs2Plan;
                            0 (default): two passes of 64-point columns (measured faster on GB300) */
} fftj_plan_opts_t;

int fftj_plan_c2c_ex(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch,
                     int64_t idist, int64_t odist, int dir, double scale, const fftj_plan_opts_t* opts);
int fftj_plan_r2c_ex(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch,
                     int64_t idist, int64_t odist, const fftj_plan_opts_t* opts);
int fftj_plan_c2r_ex(fftj_plan* out, int dtype, int rank, const int64_t* dims, int64_t batch,
                     int64_t idist, int64_t odist, int normalized, const fftj_plan_opts_t* opts);

/* Length of the feature vector fftj_plan_features writes. */
#define FFTJ_NFEATURES 28

/*
 * Cost-model features of a plan's schedule (FFTJ_NFEATURES floats): sizes,
 * dtype, kind, route, per-pass radix / tile / threads / CTAs, bytes moved.
 * Works on dry plans. Used by the learned planner to score candidates.
 */
int fftj_plan_features(fftj_plan plan, float* out, int cap);

/*
 * Autotuner (no counterpart in the reference). A query names one transform
 * problem; its candidates are the distinct schedules of a grid of
 * fftj_plan_opts_t values (dry-planned, deduplicated by schedule hash; the
 * default schedule is candidate 0).
 */
typedef struct {
  int32_t kind;     /* 0 c2c, 1 r2c, 2 c2r (irfft) */
  int32_t dtype;    /* fftj_dtype */
  int32_t rank;     /* 1..3 */
  int32_t dir;      /* c2c: -1 forward, +1 backward */
  int64_t dims[3];  /* real dims for r2c/c2r */
  int64_t batch;
  double min_ms;    /* minimum timed region per trial (0 = 0.3 ms) */
  int32_t trials;   /* timed trials per candidate, best kept (0 = 3) */
  int32_t reserved;
} fftj_tune_query_t;

/* Plan a query with the given options (NULL = default). */
int fftj_tune_plan(const fftj_tune_query_t* q, const fftj_plan_opts_t* opts, fftj_plan* out);
/* Distinct candidate schedules of a query (up to cap); *count = how many. */
int fftj_tune_candidates(const fftj_tune_query_t* q, fftj_plan_opts_t* out, int cap, int* count);
/*
 * Time candidates on the GPU: plans built in parallel on host threads, each
 * timed with CUDA events on `stream` (best of q->trials trials of
 * back-to-back executions); ms_out[i] = milliseconds per execution
 * (HUGE_VAL if candidate i cannot be planned). Allocates its own buffers.
 */
int fftj_tune_measure(const fftj_tune_query_t* q, const fftj_plan_opts_t* cands, int ncand, double* ms_out,
                      void* stream);
/* Exhaustive autotune: candidates + measurement; the fastest schedule. */
int fftj_autotune(const fftj_tune_query_t* q, fftj_plan_opts_t* best, double* best_ms);

/*
 * Learned cost model (no counterpart in the reference): an MLP in_dim -> 64
 * -> 64 -> 1 (ReLU, FP32) whose training (forward, backward, Adam) and
 * inference run as this library's own CUDA kernels. Host arrays in/out;
 * X is row-major n x in_dim. Parameters flattened as W1[64][in_dim], b1[64],
 * W2[64][64], b2[64], w3[64], b3.
 */
typedef struct fftj_mlp_s* fftj_mlp;
int fftj_mlp_create(fftj_mlp* out, int in_dim, uint64_t seed); /* He-uniform init, in_dim <= 32 */
int fftj_mlp_destroy(fftj_mlp m);
int fftj_mlp_num_params(fftj_mlp m, int64_t* count);
int fftj_mlp_get_params(fftj_mlp m, float* host, int64_t count);
int fftj_mlp_set_params(fftj_mlp m, const float* host, int64_t count);
/* Gradient of mean((f(X) - y)^2) over all n rows; *loss = that mean. */
int fftj_mlp_grad(fftj_mlp m, const float* X, const float* y, int64_t n, float* grad, double* loss);
/* Minibatch Adam for `epochs` passes (each epoch one replayed CUDA graph). */
int fftj_mlp_train(fftj_mlp m, const float* X, const float* y, int64_t n, int epochs, int minibatch, float lr,
                   uint64_t seed, double* final_loss);
int fftj_mlp_predict(fftj_mlp m, const float* X, int64_t n, float* out);

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
 * Plan from host-built tables: the caller (FFTJ's Julia planner) computes the
 * twiddles and resampling weights, the library uploads them and derives every
 * device table from them (no trigonometry of its own). Replaces the table
 * construction of src/plan.jl:66-95 (make_stage twiddles from sincospi) and
 * src/resample.jl:202-256 (_resample_parts) for 1-D complex plans.
 *   omega: 2*N doubles, re/im of exp(dir * 2 pi i e / N) for e < N.
 *   13-smooth n: N = n, rs = NULL; `scale` multiplies the result.
 *   otherwise:   resampling with the caller's tables, N = rs->m; the scale
 *                is folded into rs->corr (as _resample_parts does) and the
 *                `scale` argument is ignored.
 */
typedef struct {
  int64_t m;           /* resampled grid length: 13-smooth, >= n */
  int64_t w;           /* interpolation taps per output (1..64) */
  const double* corr;  /* n deconvolution factors, scale included */
  const double* wt;    /* n * w interpolation weights */
  const int32_t* l0;   /* n first grid rows (in [-m, m), wrapping mod m) */
} fftj_resample_tables_t;

int fftj_plan_c2c_from_tables(fftj_plan* out, int dtype, int64_t n, int64_t batch, int dir, double scale,
                              const double* omega, int64_t N, const fftj_resample_tables_t* rs);

/*
 * Apply a plan: FFTJ's p(y, x) / mul!(y, p, x) / p * x (src/api.jl:34-55,
 * src/plan.jl:359-396). d_in, d_out: device pointers; stream: a
 * cudaStream_t (NULL = legacy default stream). Asynchronous; no allocation.
 */
int fftj_execute(fftj_plan plan, const void* d_in, void* d_out, void* stream);

/*
 * Time each op (pass or elementwise kernel) of a plan: `reps` executions on
 * `stream`, CUDA events between consecutive ops; ms[i] = mean milliseconds
 * of op i (cap >= the plan's op count, fftj_plan_info_t.nops). No
 * counterpart in the reference (a measurement aid: per-pass HBM rates).
 * Needs d_in != d_out.
 */
int fftj_profile_ops(fftj_plan plan, const void* d_in, void* d_out, void* stream, int reps, float* ms, int cap);

/* Size and algorithm of a plan (FFTJ: size(p) and the plan type). */
int fftj_plan_get_info(fftj_plan plan, fftj_plan_info_t* info);

/*
 * Pipelined passes (F32 power-of-two passes of multi-pass transforms) wait
 * for their tiles' tensor copies with a bounded wait. fftj_plan_status
 * synchronises `stream` and returns FFTJ_ERR_TIMEOUT if a wait of an earlier
 * execution gave up (the status is then cleared). After such a timeout the
 * CTA waits, again bounded, for the copies it issued before it exits; the
 * plan's output is then incomplete. If even those copies never landed, the
 * CTA exited with copies into shared memory in flight, which can disturb
 * other work on the GPU: the error message says so, and the caller should
 * treat every result produced on the stream since its previous status check
 * as lost. No counterpart in the reference (host code has no device waits).
 */
int fftj_plan_status(fftj_plan plan, void* stream);
/* Bound of each such wait in nanoseconds (default 1e9). */
int fftj_plan_set_wait_limit(fftj_plan plan, uint64_t ns);
/* Test hook: tile barriers expect `extra_bytes` more than their copies
 * deliver, so every wait runs out (0 restores normal operation). */
int fftj_plan_debug_stall(fftj_plan plan, int extra_bytes);

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
 * as real-time loops that forbid allocation once they run (an allocation can
 * block on the driver for an unbounded time), and hosts that own all device
 * memory through their own pool and cannot hand a plan its workspace. It
 * creates no plan and calls no
 * cudaMalloc, cudaFree or other allocating routine: its scratch is a
 * file-scope static device array of 64 MiB (1 MiB of twiddle tables,
 * regenerated on the device on every call, and 63 MiB for the intermediate
 * of a two-pass transform) that every GPU loading the library holds until
 * exit. Limits: n 13-smooth and done in one or two passes (n <= 2^20 F32, 2^18 F64), and
 * for two passes batch * n * sizeof(complex) <= 63 MiB; larger requests
 * return FFTJ_ERR_ARG / FFTJ_ERR_UNSUPPORTED with a message. d_in/d_out hold
 * batch dense transforms; in == out is allowed. The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) and keeps it;
 * a device reset (cudaDeviceReset) after that first call is not supported:
 * the kept address would be stale. A CUDA error already pending on the calling thread is
 * reported as FFTJ_ERR_CUDA and left pending. All calls share the one array: calls that
 * overlap on the GPU (other streams, other threads) race and must be
 * serialised by the caller. Nothing in the array needs to start at zero.
 */
int fftj_execute_noalloc_c2c(int dtype, int64_t n, int64_t batch, int dir, double scale, const void* d_in,
                             void* d_out, void* stream);

/*
 * Groups: many plans executed as one unit (no counterpart in the reference,
 * which runs one plan per call). A group binds distinct plans to their
 * buffers at creation; each execution runs all of them on `stream`.
 *   FFTJ_GROUP_STREAM      the plans' kernels launched back to back;
 *   FFTJ_GROUP_GRAPH       the same launches captured once as a CUDA graph
 *                          with the plans on parallel branches;
 *   FFTJ_GROUP_PERSISTENT  one persistent kernel draining a device queue of
 *                          (op, tile range) items with bounded dependency
 *                          waits, captured with a small queue-reset kernel
 *                          as a CUDA graph (2 kernels per execution). Every
 *                          pass must use <= 256 threads per CTA (plan with
 *                          opts.threads_max = 256).
 * Plans must outlive the group and must not run elsewhere while it runs.
 */
typedef struct fftj_group_s* fftj_group;
typedef enum { FFTJ_GROUP_STREAM = 0, FFTJ_GROUP_GRAPH = 1, FFTJ_GROUP_PERSISTENT = 2 } fftj_group_mode;
typedef struct {
  int mode;
  int nplans;
  int nops;        /* ops over all plans */
  int nitems;      /* queue items (persistent) */
  int ctas;        /* persistent CTAs (one per resident slot) */
  int smem_bytes;  /* dynamic shared memory of the persistent kernel */
  int branches;    /* parallel graph branches (graph mode) */
  int kernels;     /* kernel launches per execution */
} fftj_group_info_t;

int fftj_group_create(fftj_group* out, int count, const fftj_plan* plans, const void* const* d_in,
                      void* const* d_out, int mode);
int fftj_group_execute(fftj_group g, void* stream);
/* Waits for the last execution; FFTJ_ERR_TIMEOUT if a persistent wait gave up. */
int fftj_group_status(fftj_group g);
int fftj_group_get_info(fftj_group g, fftj_group_info_t* info);
/* Spin limit of each persistent dependency wait (default 2e6 polls, ~1 s). */
int fftj_group_set_wait_limit(fftj_group g, uint32_t spins);
/* Test hook: op `op` of a persistent group waits for a count that is never
 * reached, so its waits run out (to exercise the timeout path). */
int fftj_group_debug_stall(fftj_group g, int op);
int fftj_group_destroy(fftj_group g);

#ifdef __cplusplus
}
#endif

#endif /* FFTJ_H */
