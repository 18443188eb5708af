// Exhaustive schedule autotuner (no counterpart in the reference: FFTJ picks
// its schedule from fixed vector-width and cache thresholds,
// src/plan.jl:105-151, src/fourstep.jl:166-230).
//
// A query (kind, dtype, dims, batch) has a set of candidate schedules: the
// grid of fftj_plan_opts_t values (tile, extra passes, radix order, threads
// per column, route for non-smooth lengths), reduced to the distinct launch
// schedules by planning each one dry and comparing schedule hashes. The
// tuner builds the candidates' plans on host threads in parallel, then times
// each on one stream with CUDA events: warm-up executions, then trials of
// back-to-back executions long enough to cover launch latency; the figure is
// the best trial's time per execution. The fastest candidate is the
// exhaustive choice that the learned cost model is trained on and scored against.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fftj.h"
#include "fftj_internal.h"

namespace {

int tune_fail(int code, const char* msg) {
  fftj::set_error(msg);
  return code;
}

int64_t query_n(const fftj_tune_query_t* q) {
  int64_t n = 1;
  for (int i = 0; i < q->rank; ++i) n *= q->dims[i];
  return n;
}

int check_query(const fftj_tune_query_t* q) {
  if (!q) return tune_fail(FFTJ_ERR_ARG, "null query");
  if (q->kind < 0 || q->kind > 2) return tune_fail(FFTJ_ERR_ARG, "query kind must be 0 (c2c), 1 (r2c) or 2 (c2r)");
  if (q->rank < 1 || q->rank > 3) return tune_fail(FFTJ_ERR_ARG, "query rank must be 1..3");
  for (int i = 0; i < q->rank; ++i)
    if (q->dims[i] < 1) return tune_fail(FFTJ_ERR_ARG, "query dims must be >= 1");
  if (q->batch < 1) return tune_fail(FFTJ_ERR_ARG, "query batch must be >= 1");
  return FFTJ_OK;
}

bool odd_nonsmooth(int64_t n) {
  int64_t r = n;
  for (int p : {2, 3, 5, 7, 11, 13})
    while (r % p == 0) r /= p;
  return r != 1;
}

}  // namespace

extern "C" {

int fftj_tune_plan(const fftj_tune_query_t* q, const fftj_plan_opts_t* opts, fftj_plan* out) {
  if (int rc = check_query(q)) return rc;
  const int dir = q->dir == 1 ? 1 : -1;
  switch (q->kind) {
    case 0: return fftj_plan_c2c_ex(out, q->dtype, q->rank, q->dims, q->batch, 0, 0, dir, 1.0, opts);
    case 1: return fftj_plan_r2c_ex(out, q->dtype, q->rank, q->dims, q->batch, 0, 0, opts);
    default: return fftj_plan_c2r_ex(out, q->dtype, q->rank, q->dims, q->batch, 0, 0, 1, opts);
  }
}

int fftj_tune_candidates(const fftj_tune_query_t* q, fftj_plan_opts_t* out, int cap, int* count) {
  if (int rc = check_query(q)) return rc;
  if (!out || !count || cap < 1) return tune_fail(FFTJ_ERR_ARG, "null output or cap < 1");
  const int64_t n = query_n(q);
  // a non-smooth length anywhere in the transform makes the route a knob
  bool nonsmooth = false;
  for (int i = 0; i < q->rank; ++i) nonsmooth = nonsmooth || odd_nonsmooth(q->dims[i]);
  (void)n;
  std::vector<uint64_t> seen;
  int k = 0;
  const int tiles[] = {0, 2048};
  const int routes_smooth[] = {0};
  const int routes_ns[] = {0, 1, 2};
  const int* routes = nonsmooth ? routes_ns : routes_smooth;
  const int nroutes = nonsmooth ? 3 : 1;
  for (int ri = 0; ri < nroutes; ++ri)
    for (int extra = 0; extra <= 1; ++extra)
      for (int order = 0; order <= 1; ++order)
        for (int tf : {0, 2})
          for (int tile : tiles) {
            fftj_plan_opts_t o;
            std::memset(&o, 0, sizeof(o));
            o.tile = tile;
            o.extra_passes = extra;
            o.order = order;
            o.tf_mult = tf;
            o.route = routes[ri];
            o.dry = 1;
            fftj_plan p = nullptr;
            if (fftj_tune_plan(q, &o, &p) != FFTJ_OK) continue;
            fftj_plan_info_t info;
            fftj_plan_get_info(p, &info);
            fftj_plan_destroy(p);
            if (std::find(seen.begin(), seen.end(), info.schedule_hash) != seen.end()) continue;
            seen.push_back(info.schedule_hash);
            if (k < cap) {
              o.dry = 0;
              out[k] = o;
            }
            k++;
          }
  *count = std::min(k, cap);
  fftj::set_error("");
  return k == 0 ? tune_fail(FFTJ_ERR_UNSUPPORTED, "no schedule plans this query") : FFTJ_OK;
}

int fftj_tune_measure(const fftj_tune_query_t* q, const fftj_plan_opts_t* cands, int ncand, double* ms_out,
                      void* stream) {
  if (int rc = check_query(q)) return rc;
  if (!cands || !ms_out || ncand < 1) return tune_fail(FFTJ_ERR_ARG, "null candidates/output or ncand < 1");
  const int64_t n = query_n(q);
  const size_t esz = q->dtype == FFTJ_F64 ? 16 : 8;
  // upper bound of either side of any kind: batch * (n + 2 * rows) complex
  const size_t bytes = (size_t)q->batch * (size_t)(n + 2 * (n / q->dims[0]) + 2) * esz;
  void *d_in = nullptr, *d_out = nullptr;
  if (cudaMalloc(&d_in, bytes) != cudaSuccess || cudaMalloc(&d_out, bytes) != cudaSuccess) {
    cudaFree(d_in);
    return tune_fail(FFTJ_ERR_CUDA, "tuner buffer allocation failed");
  }
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemsetAsync(d_in, 0, bytes, st);
  cudaMemsetAsync(d_out, 0, bytes, st);

  // candidates' plans, built in parallel (planning is host work: tables)
  std::vector<fftj_plan> plans(ncand, nullptr);
  int dev = 0;
  cudaGetDevice(&dev);
  {
    const int nth = std::max(1, std::min<int>(ncand, (int)std::min(8u, std::max(1u, std::thread::hardware_concurrency()))));
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t)
      th.emplace_back([&, t]() {
        cudaSetDevice(dev);
        for (int i = t; i < ncand; i += nth)
          if (fftj_tune_plan(q, &cands[i], &plans[i]) != FFTJ_OK) plans[i] = nullptr;
      });
    for (auto& x : th) x.join();
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const double min_ms = q->min_ms > 0 ? q->min_ms : 0.3;
  const int trials = q->trials > 0 ? q->trials : 3;
  int rc = FFTJ_OK;
  for (int i = 0; i < ncand; ++i) {
    ms_out[i] = HUGE_VAL;
    fftj_plan p = plans[i];
    if (!p) continue;
    bool ok = true;
    for (int w = 0; w < 2 && ok; ++w) ok = fftj_execute(p, d_in, d_out, st) == FFTJ_OK;
    float t1 = 0;
    ok = ok && cudaEventRecord(e0, st) == cudaSuccess && fftj_execute(p, d_in, d_out, st) == FFTJ_OK &&
         cudaEventRecord(e1, st) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
         cudaEventElapsedTime(&t1, e0, e1) == cudaSuccess;
    if (!ok) {
      rc = tune_fail(FFTJ_ERR_CUDA, "tuner execution failed");
      break;
    }
    const int reps = (int)std::min<double>(256.0, std::max<double>(1.0, std::ceil(min_ms / std::max<double>(t1, 1e-4))));
    double best = HUGE_VAL;
    for (int tr = 0; tr < trials && ok; ++tr) {
      ok = cudaEventRecord(e0, st) == cudaSuccess;
      for (int r = 0; r < reps && ok; ++r) ok = fftj_execute(p, d_in, d_out, st) == FFTJ_OK;
      float ms = 0;
      ok = ok && cudaEventRecord(e1, st) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
           cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
      if (ok) best = std::min(best, (double)ms / reps);
    }
    if (!ok) {
      rc = tune_fail(FFTJ_ERR_CUDA, "tuner execution failed");
      break;
    }
    ms_out[i] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (auto p : plans) fftj_plan_destroy(p);
  cudaStreamSynchronize(st);
  cudaFree(d_in);
  cudaFree(d_out);
  if (rc == FFTJ_OK) fftj::set_error("");
  return rc;
}

int fftj_autotune(const fftj_tune_query_t* q, fftj_plan_opts_t* best, double* best_ms) {
  if (!best) return tune_fail(FFTJ_ERR_ARG, "null output");
  std::vector<fftj_plan_opts_t> c(64);
  int k = 0;
  if (int rc = fftj_tune_candidates(q, c.data(), (int)c.size(), &k)) return rc;
  std::vector<double> ms(k);
  if (int rc = fftj_tune_measure(q, c.data(), k, ms.data(), nullptr)) return rc;
  int bi = 0;
  for (int i = 1; i < k; ++i)
    if (ms[i] < ms[bi]) bi = i;
  *best = c[bi];
  if (best_ms) *best_ms = ms[bi];
  return FFTJ_OK;
}

}  // extern "C"
