// Many plans as one unit of work (no counterpart in the reference: FFTJ runs
// one plan per call and batches only by looping). A group binds a list of
// distinct plans to their input/output buffers and executes them in one of
// three forms:
//
//  STREAM      every plan's kernels launched back to back on the stream;
//  GRAPH       the same launches captured once as a CUDA graph whose plans
//              sit on parallel branches (independent transforms run
//              concurrently), replayed by one cudaGraphLaunch;
//  PERSISTENT  one persistent kernel (one CTA per resident slot) that drains
//              a device work queue of (op, tile range) items, captured with
//              a small kernel that resets the queue as a CUDA graph. Items are queued level by
//              level (every plan's first op, then every plan's second op,
//              ...); an item of op k of a plan waits until all tiles of op
//              k-1 of that plan are done. A CTA claims items in queue order
//              with an atomic counter, so every item it waits for was claimed
//              earlier by a running CTA: the waits always end. Each wait is
//              still bounded (a spin limit with a back-off sleep); a wait that
//              runs out records an error the host reads (fftj_group_status),
//              counts its item as done and moves on, so the kernel always
//              finishes.
//
// Ops run in the persistent kernel through the same device code as their
// own kernels: the runtime-recipe pass body (pass_tile) and the elementwise
// bodies (elementwise.cuh), with L2-coherent loads because their inputs were
// written earlier in the same launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "elementwise.cuh"
#include "pass_common.cuh"
#include "plan_internal.h"

namespace fftj {

constexpr int kGroupThreads = 256;  // CTA size of the persistent kernel
constexpr int kEwTile = 256;        // elements (solve: chunks) per elementwise tile
#ifndef FFTJ_GROUP_SOLVE_K
#define FFTJ_GROUP_SOLVE_K 4
#endif
constexpr int kGroupSolveK = FFTJ_GROUP_SOLVE_K;  // rows per block of the banded solve (registers)

struct alignas(16) GroupOp {
  int32_t kind, f64, dir, load_op;
  int32_t B, dep;            // solve band; op this op waits for (-1: none)
  uint32_t dep_need, ntiles; // tiles of dep that must be done; tiles of this op
  const void* src;
  void* dst;
  PassParams pp;
  InterpParams ip;
  RealPostParams rp;
  CopyParams cp;
  SolveParams sv;
};
static_assert(sizeof(GroupOp) % 16 == 0, "GroupOp is copied to shared memory as int4");

struct GroupItem {
  int32_t op;
  uint32_t t0, t1;
  int32_t pad;
};

// ctl[0]: queue head, ctl[1]: error flag, ctl[2]: op of the first failed
// wait, ctl[3]: spin limit; done[op] follows at ctl + 4.
constexpr int kCtlWords = 4;

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// LOADOP: LOAD_PLAIN for the passes that read plain data (most of them: a
// function of their own keeps the other load ops' code and registers out),
// LOAD_RUNTIME for first passes with a fused load op
template <typename T, int DIR, int LOADOP>
__device__ __noinline__ void group_pass(const PassParams& pp, const void* src, void* dst, uint32_t t0, uint32_t t1,
                                        int tid) {
  for (uint32_t t = t0; t < t1; ++t) {
    pass_tile<T, DIR, LOADOP, RuntimeRecipe, true>(pp, src, reinterpret_cast<Cx<Hs<T>>*>(dst), t, tid, pp.threads);
    __syncthreads();  // the next tile reuses the shared buffer
  }
}
template <typename T, int DIR>
__device__ __forceinline__ void group_pass_any(const PassParams& pp, const void* src, void* dst, uint32_t t0,
                                               uint32_t t1, int tid) {
  if (pp.load_op == LOAD_PLAIN) group_pass<T, DIR, LOAD_PLAIN>(pp, src, dst, t0, t1, tid);
  else group_pass<T, DIR, LOAD_RUNTIME>(pp, src, dst, t0, t1, tid);
}

// the solve with factors rebuilt per call, out of line (keeps the other
// elementwise bodies' registers)
template <typename T>
__device__ __noinline__ void group_solve_fly(const GroupOp& op, int64_t idx) {
  const Cx<T>* src = reinterpret_cast<const Cx<T>*>(op.src);
  Cx<T>* dst = reinterpret_cast<Cx<T>*>(op.dst);
  if (op.B == 1) solve_fly_at<T, 1, true>(op.sv, src, dst, idx);
  else if (op.B == 2) solve_fly_at<T, 2, true>(op.sv, src, dst, idx);
  else solve_fly_at<T, 3, true>(op.sv, src, dst, idx);
}

// Each elementwise kind runs its item's tiles in a function of its own, so
// that each gets its own register allocation (the banded solve needs many
// more than a copy).
template <typename T>
__device__ __noinline__ void group_interp(const GroupOp& op, uint32_t t0, uint32_t t1, int tid) {
  for (uint32_t t = t0; t < t1; ++t)
    interp_at<T, true>(op.ip, reinterpret_cast<const Cx<T>*>(op.src), reinterpret_cast<Cx<T>*>(op.dst),
                       (int64_t)t * kEwTile + tid);
}
template <typename T>
__device__ __noinline__ void group_rpost(const GroupOp& op, uint32_t t0, uint32_t t1, int tid) {
  for (uint32_t t = t0; t < t1; ++t)
    real_post_at<T, true>(op.rp, reinterpret_cast<const Cx<T>*>(op.src), reinterpret_cast<Cx<T>*>(op.dst),
                          (int64_t)t * kEwTile + tid);
}
template <typename T>
__device__ __noinline__ void group_copy(const GroupOp& op, uint32_t t0, uint32_t t1, int tid) {
  for (uint32_t t = t0; t < t1; ++t) copy_at<T, true>(op.cp, op.src, op.dst, (int64_t)t * kEwTile + tid);
}
template <typename T, int B>
__device__ __noinline__ void group_solve(const GroupOp& op, uint32_t t0, uint32_t t1, int tid) {
  for (uint32_t t = t0; t < t1; ++t)
    solve_at<T, B, true, kGroupSolveK>(op.sv, reinterpret_cast<const Cx<T>*>(op.src),
                                       reinterpret_cast<Cx<T>*>(op.dst), (int64_t)t * kEwTile + tid);
}
template <typename T>
__device__ __forceinline__ void group_elementwise(const GroupOp& op, uint32_t t0, uint32_t t1, int tid) {
  switch (op.kind) {
    case OP_INTERP: group_interp<T>(op, t0, t1, tid); break;
    case OP_RPOST: group_rpost<T>(op, t0, t1, tid); break;
    case OP_COPY: group_copy<T>(op, t0, t1, tid); break;
    case OP_SOLVE:
      if (op.sv.fly) {
        for (uint32_t t = t0; t < t1; ++t) group_solve_fly<T>(op, (int64_t)t * kEwTile + tid);
      } else if (op.B == 1) {
        group_solve<T, 1>(op, t0, t1, tid);
      } else if (op.B == 2) {
        group_solve<T, 2>(op, t0, t1, tid);
      } else {
        group_solve<T, 3>(op, t0, t1, tid);
      }
      break;
    default: break;
  }
}

// Zeroes the queue head, the error word, the failed op and every done
// counter before an execution. A kernel rather than memset nodes: memsets
// can be queued on a copy engine behind multi-gigabyte host copies of other
// streams, holding the execution back until those copies finish.
__global__ void k_group_reset(uint32_t* ctl, int nops) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 3) ctl[i] = 0;
  if (i < nops) ctl[kCtlWords + i] = 0;
}

__global__ void __launch_bounds__(kGroupThreads, 2)
    k_group(const GroupOp* __restrict__ ops, const GroupItem* __restrict__ items, int nitems, uint32_t* ctl) {
  __shared__ __align__(16) unsigned char sop_raw[sizeof(GroupOp)];
  GroupOp& sop = *reinterpret_cast<GroupOp*>(sop_raw);
  __shared__ int s_item;
  __shared__ int s_skip;
  uint32_t* done = ctl + kCtlWords;
  const int tid = threadIdx.x;
  const uint32_t limit = ctl[3];
  for (;;) {
    if (tid == 0) s_item = (int)atomicAdd(&ctl[0], 1u);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) return;
    const GroupItem item = items[it];
    {
      const int4* s = reinterpret_cast<const int4*>(ops + item.op);
      int4* d = reinterpret_cast<int4*>(&sop);
      for (int i = tid; i < (int)(sizeof(GroupOp) / 16); i += blockDim.x) d[i] = s[i];
    }
    if (tid == 0) {
      int skip = 0;
      const int dep = ops[item.op].dep;
      if (dep >= 0) {
        const uint32_t need = ops[item.op].dep_need;
        uint32_t spins = 0;
        while (ld_acquire_u32(done + dep) < need) {
          if (++spins > limit) {
            skip = 1;
            if (atomicExch(&ctl[1], 1u) == 0u) atomicExch(&ctl[2], (uint32_t)item.op);
            break;
          }
          __nanosleep(256);
        }
      }
      s_skip = skip;
    }
    __syncthreads();
    if (!s_skip) {
      if (sop.kind == OP_PASS) {
        if (sop.f64) {  // block fixed point (group creation rejects FP64-butterfly passes)
          if (sop.dir < 0) group_pass_any<Fx, -1>(sop.pp, sop.src, sop.dst, item.t0, item.t1, tid);
          else group_pass_any<Fx, 1>(sop.pp, sop.src, sop.dst, item.t0, item.t1, tid);
        } else {
          if (sop.dir < 0) group_pass_any<float, -1>(sop.pp, sop.src, sop.dst, item.t0, item.t1, tid);
          else group_pass_any<float, 1>(sop.pp, sop.src, sop.dst, item.t0, item.t1, tid);
        }
      } else if (sop.f64) {
        group_elementwise<double>(sop, item.t0, item.t1, tid);
      } else {
        group_elementwise<float>(sop, item.t0, item.t1, tid);
      }
    }
    __syncthreads();  // the item's stores are issued; sop and s_item are reused
    if (tid == 0) {
      __threadfence();
      atomicAdd(done + item.op, item.t1 - item.t0);
    }
  }
}

}  // namespace fftj

using namespace fftj;

struct fftj_group_s {
  int mode = 0;
  std::vector<fftj_plan> plans;
  std::vector<const void*> in;
  std::vector<void*> out;
  int nops = 0, nitems = 0, ctas = 0, branches = 0;
  size_t smem = 0;
  GroupOp* d_ops = nullptr;
  GroupItem* d_items = nullptr;
  uint32_t* d_ctl = nullptr;
  std::vector<GroupOp> h_ops;
  cudaStream_t cap = nullptr;
  std::vector<cudaStream_t> br;
  std::vector<cudaEvent_t> ev;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t last = nullptr;
  bool ran = false;
  ~fftj_group_s() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto e : ev) cudaEventDestroy(e);
    for (auto s : br) cudaStreamDestroy(s);
    if (cap) cudaStreamDestroy(cap);
    cudaFree(d_ops);
    cudaFree(d_items);
    cudaFree(d_ctl);
  }
};

namespace {

int gfail(int code, const std::string& msg) {
  set_error(msg.c_str());
  return code;
}

uint32_t op_tiles(const Op& op) {
  auto ew = [](int64_t total) { return (uint32_t)((total + kEwTile - 1) / kEwTile); };
  switch (op.kind) {
    case OP_PASS: return op.pp.tiles_q * op.pp.tiles_p * op.pp.tiles_b;
    case OP_INTERP: return ew(op.ip.n * op.ip.nbatch * std::max<int64_t>(op.ip.inner, 1));
    case OP_RPOST: return ew((op.rp.h / 2 + 1) * op.rp.nbatch);
    case OP_COPY: return ew(op.cp.n * op.cp.nbatch);
    case OP_SOLVE: return ew(op.sv.nbatch * op.sv.nchunk);
  }
  return 0;
}

// tiles per queue item: about 16K elements of F32 / 4K of ComplexF64 pass
// work (four / two tiles of the default size), 2K elementwise elements, one
// tile of solve chunks. All passes at 2K / 4K / 8K / 16K elements: 113.5 /
// 109.8-111.1 / 111.0 / 116.3 ms for the uneven batch; F32 at 4K / 8K / 16K
// with ComplexF64 at 4K: 15.9 / 13.7 / 13.3 ms of F32 c2c (107.1 ms step).
uint32_t item_chunk(const Op& op, bool f64) {
  const int64_t elems = f64 ? 4096 : 16384;
  if (op.kind == OP_PASS) return (uint32_t)std::max<int64_t>(1, elems / ((int64_t)op.pp.NB * op.pp.R));
  if (op.kind == OP_SOLVE) return 1;
  return 8;
}

int build_persistent(fftj_group_s* g) {
  // device op table, level by level
  std::vector<int> first(g->plans.size());
  size_t maxlev = 0;
  for (size_t p = 0; p < g->plans.size(); ++p) {
    fftj_plan P = g->plans[p];
    first[p] = (int)g->h_ops.size();
    maxlev = std::max(maxlev, P->ops.size());
    void* bufs[4] = {const_cast<void*>(g->in[p]), g->out[p], P->ws[0].p, P->ws[1].p};
    for (size_t j = 0; j < P->ops.size(); ++j) {
      const Op& op = P->ops[j];
      GroupOp go;
      std::memset(&go, 0, sizeof(go));
      go.kind = op.kind;
      go.f64 = P->dtype == FFTJ_F64;
      go.dir = op.dir;
      go.load_op = op.kind == OP_PASS ? op.pp.load_op : 0;
      go.B = op.sv.B;
      go.dep = j ? (int)g->h_ops.size() - 1 : -1;
      go.dep_need = j ? g->h_ops.back().ntiles : 0;
      go.ntiles = op_tiles(op);
      go.src = bufs[op.src];
      go.dst = bufs[op.dst];
      go.pp = op.pp;
      go.ip = op.ip;
      go.rp = op.rp;
      go.cp = op.cp;
      go.sv = op.sv;
      if (op.kind == OP_PASS) {
        if (op.pp.threads > kGroupThreads)
          return gfail(FFTJ_ERR_UNSUPPORTED,
                       "persistent group: a pass uses " + std::to_string(op.pp.threads) +
                           " threads per CTA; plan it with opts.threads_max = 256");
        if (go.f64 && !op.pp.fx)
          return gfail(FFTJ_ERR_UNSUPPORTED,
                       "persistent group: ComplexF64 plans with FP64 butterflies (opts.f64_arith = 1) run "
                       "outside persistent groups");
        const size_t esz = go.f64 ? 16 : 8;
        // passes run the run-time-radix body, which ping-pongs between two
        // tile buffers
        g->smem = std::max(g->smem, 2 * (size_t)op.pp.smem_elems * esz + (size_t)op.pp.fx_cols * sizeof(int));
      }
      g->h_ops.push_back(go);
    }
  }
  g->nops = (int)g->h_ops.size();
  // queue: level-major; within a level, by device code, then plans with
  // more work first
  std::vector<size_t> order(g->plans.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    return g->plans[a]->n * g->plans[a]->batch > g->plans[b]->n * g->plans[b]->batch;
  });
  std::vector<GroupItem> items;
  for (size_t lev = 0; lev < maxlev; ++lev) {
    // the level's ops grouped by the device code they run (op kind, dtype,
    // direction, plain or fused load), larger plans first in each: CTAs
    // that run at the same time then run the same functions (fewer
    // instruction-cache misses; the uneven batch's step 115.9 -> 113.5 ms)
    std::vector<size_t> lo(order);
    auto code = [&](size_t p) {
      if (lev >= g->plans[p]->ops.size()) return 1 << 20;
      const GroupOp& o = g->h_ops[first[p] + (int)lev];
      return ((o.kind * 2 + o.f64) * 2 + (o.dir > 0)) * 2 + (o.load_op != LOAD_PLAIN);
    };
    std::stable_sort(lo.begin(), lo.end(), [&](size_t a, size_t b) { return code(a) < code(b); });
    for (size_t p : lo) {
      fftj_plan P = g->plans[p];
      if (lev >= P->ops.size()) continue;
      const int oi = first[p] + (int)lev;
      const uint32_t nt = g->h_ops[oi].ntiles, ch = item_chunk(P->ops[lev], P->dtype == FFTJ_F64);
      for (uint32_t t = 0; t < nt; t += ch) items.push_back(GroupItem{oi, t, std::min(nt, t + ch), 0});
    }
  }
  g->nitems = (int)items.size();

  int dev = 0, sms = 0, optin = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return gfail(FFTJ_ERR_CUDA, "persistent group: device query failed");
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, (const void*)k_group) != cudaSuccess)
    return gfail(FFTJ_ERR_CUDA, "persistent group: kernel attribute query failed");
  const int maxdyn = optin - (int)fa.sharedSizeBytes;
  if (maxdyn <= 0 || g->smem > (size_t)maxdyn)
    return gfail(FFTJ_ERR_UNSUPPORTED, "persistent group: a pass tile exceeds shared memory");
  if (cudaFuncSetAttribute((const void*)k_group, cudaFuncAttributeMaxDynamicSharedMemorySize, maxdyn) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_group, kGroupThreads, g->smem) != cudaSuccess ||
      per_sm < 1)
    return gfail(FFTJ_ERR_CUDA, "persistent group: kernel configuration failed");
  g->ctas = std::max(1, std::min(g->nitems, per_sm * sms));

  const size_t ctl_bytes = (kCtlWords + (size_t)g->nops) * sizeof(uint32_t);
  if (cudaMalloc(&g->d_ops, g->h_ops.size() * sizeof(GroupOp)) != cudaSuccess ||
      cudaMalloc(&g->d_items, std::max<size_t>(1, items.size()) * sizeof(GroupItem)) != cudaSuccess ||
      cudaMalloc(&g->d_ctl, ctl_bytes) != cudaSuccess)
    return gfail(FFTJ_ERR_CUDA, "persistent group: allocation failed");
  if (cudaMemcpy(g->d_ops, g->h_ops.data(), g->h_ops.size() * sizeof(GroupOp), cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(g->d_items, items.data(), items.size() * sizeof(GroupItem), cudaMemcpyHostToDevice) != cudaSuccess)
    return gfail(FFTJ_ERR_CUDA, "persistent group: upload failed");
  // one execution = reset the queue head, error word and done counters
  // (the spin limit word is written once, here), then the kernel
  const uint32_t ctl0[kCtlWords] = {0, 0, 0, 2000000u};
  if (cudaMemcpy(g->d_ctl, ctl0, sizeof(ctl0), cudaMemcpyHostToDevice) != cudaSuccess)
    return gfail(FFTJ_ERR_CUDA, "persistent group: upload failed");
  if (cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return gfail(FFTJ_ERR_CUDA, "persistent group: graph capture failed");
  const int nreset = std::max(g->nops, 3);
  k_group_reset<<<(nreset + 255) / 256, 256, 0, g->cap>>>(g->d_ctl, g->nops);
  k_group<<<g->ctas, kGroupThreads, g->smem, g->cap>>>(g->d_ops, g->d_items, g->nitems, g->d_ctl);
  const cudaError_t le = cudaGetLastError();
  if (cudaStreamEndCapture(g->cap, &g->graph) != cudaSuccess || le != cudaSuccess ||
      cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess)
    return gfail(FFTJ_ERR_CUDA, "persistent group: graph instantiation failed");
  return FFTJ_OK;
}

int build_graph(fftj_group_s* g) {
  g->branches = (int)std::min<size_t>(8, g->plans.size());
  for (int i = 0; i < g->branches; ++i) {
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
      return gfail(FFTJ_ERR_CUDA, "graph group: stream creation failed");
    g->br.push_back(s);
  }
  for (int i = 0; i < g->branches + 1; ++i) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
      return gfail(FFTJ_ERR_CUDA, "graph group: event creation failed");
    g->ev.push_back(e);
  }
  if (cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return gfail(FFTJ_ERR_CUDA, "graph group: capture failed");
  int rc = FFTJ_OK;
  cudaEventRecord(g->ev[g->branches], g->cap);
  for (int b = 0; b < g->branches; ++b) cudaStreamWaitEvent(g->br[b], g->ev[g->branches], 0);
  for (size_t p = 0; p < g->plans.size() && rc == FFTJ_OK; ++p)
    rc = fftj_execute(g->plans[p], g->in[p], g->out[p], g->br[p % g->branches]);
  for (int b = 0; b < g->branches; ++b) {
    cudaEventRecord(g->ev[b], g->br[b]);
    cudaStreamWaitEvent(g->cap, g->ev[b], 0);
  }
  const cudaError_t ce = cudaStreamEndCapture(g->cap, &g->graph);
  if (rc != FFTJ_OK) return rc;
  if (ce != cudaSuccess || cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess)
    return gfail(FFTJ_ERR_CUDA, "graph group: graph instantiation failed");
  return FFTJ_OK;
}

}  // namespace

extern "C" {

int fftj_group_create(fftj_group* out, int count, const fftj_plan* plans, const void* const* d_in,
                      void* const* d_out, int mode) {
  if (!out) return gfail(FFTJ_ERR_ARG, "null group pointer");
  *out = nullptr;
  if (count < 1 || !plans || !d_in || !d_out) return gfail(FFTJ_ERR_ARG, "empty group or null arrays");
  if (mode < FFTJ_GROUP_STREAM || mode > FFTJ_GROUP_PERSISTENT) return gfail(FFTJ_ERR_ARG, "unknown group mode");
  std::unique_ptr<fftj_group_s> g(new fftj_group_s());
  g->mode = mode;
  std::vector<fftj_plan> sorted(plans, plans + count);
  std::sort(sorted.begin(), sorted.end());
  if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
    return gfail(FFTJ_ERR_ARG, "a plan appears twice in a group (plans own their workspace)");
  for (int i = 0; i < count; ++i) {
    if (!plans[i] || plans[i]->dry) return gfail(FFTJ_ERR_ARG, "null or dry plan in group");
    if (!d_in[i] || !d_out[i]) return gfail(FFTJ_ERR_ARG, "null data pointer in group");
    if (mode == FFTJ_GROUP_PERSISTENT && d_in[i] == d_out[i] && plans[i]->ops.size() == 1 && !plans[i]->inplace_safe)
      return gfail(FFTJ_ERR_ARG, "persistent group: this plan needs distinct input and output buffers");
    g->plans.push_back(plans[i]);
    g->in.push_back(d_in[i]);
    g->out.push_back(d_out[i]);
  }
  for (auto P : g->plans) g->nops += (int)P->ops.size();
  int rc = FFTJ_OK;
  if (mode != FFTJ_GROUP_STREAM) {
    if (cudaStreamCreateWithFlags(&g->cap, cudaStreamNonBlocking) != cudaSuccess)
      return gfail(FFTJ_ERR_CUDA, "group: stream creation failed");
    if (mode == FFTJ_GROUP_GRAPH) {
      rc = build_graph(g.get());
    } else {
      g->nops = 0;
      rc = build_persistent(g.get());
    }
  }
  if (rc) return rc;
  *out = g.release();
  set_error("");
  return FFTJ_OK;
}

int fftj_group_execute(fftj_group g, void* stream) {
  if (!g) return gfail(FFTJ_ERR_ARG, "null group");
  cudaStream_t st = (cudaStream_t)stream;
  g->last = st;
  g->ran = true;
  if (g->mode == FFTJ_GROUP_STREAM) {
    for (size_t p = 0; p < g->plans.size(); ++p)
      if (int rc = fftj_execute(g->plans[p], g->in[p], g->out[p], st)) return rc;
    set_error("");
    return FFTJ_OK;
  }
  if (cudaGraphLaunch(g->exec, st) != cudaSuccess) return gfail(FFTJ_ERR_CUDA, "group: graph launch failed");
  set_error("");
  return FFTJ_OK;
}

int fftj_group_status(fftj_group g) {
  if (!g) return gfail(FFTJ_ERR_ARG, "null group");
  if (!g->ran) return FFTJ_OK;
  if (cudaStreamSynchronize(g->last) != cudaSuccess) return gfail(FFTJ_ERR_CUDA, "group: execution failed");
  if (g->mode != FFTJ_GROUP_PERSISTENT) return FFTJ_OK;
  uint32_t ctl[kCtlWords];
  if (cudaMemcpy(ctl, g->d_ctl, sizeof(ctl), cudaMemcpyDeviceToHost) != cudaSuccess)
    return gfail(FFTJ_ERR_CUDA, "group: status read failed");
  if (ctl[1])
    return gfail(FFTJ_ERR_TIMEOUT, "persistent group: a dependency wait gave up (op " + std::to_string(ctl[2]) +
                                       "); its items were skipped");
  set_error("");
  return FFTJ_OK;
}

int fftj_group_get_info(fftj_group g, fftj_group_info_t* info) {
  if (!g || !info) return gfail(FFTJ_ERR_ARG, "null argument");
  std::memset(info, 0, sizeof(*info));
  info->mode = g->mode;
  info->nplans = (int)g->plans.size();
  info->nops = g->nops;
  info->nitems = g->nitems;
  info->ctas = g->ctas;
  info->smem_bytes = (int)g->smem;
  info->branches = g->branches;
  info->kernels = g->mode == FFTJ_GROUP_PERSISTENT ? 2 : g->nops;  // persistent: the reset and the queue kernel
  return FFTJ_OK;
}

int fftj_group_set_wait_limit(fftj_group g, uint32_t spins) {
  if (!g) return gfail(FFTJ_ERR_ARG, "null group");
  if (g->mode != FFTJ_GROUP_PERSISTENT) return FFTJ_OK;
  if (spins < 1) return gfail(FFTJ_ERR_ARG, "wait limit must be >= 1");
  return cudaMemcpy(g->d_ctl + 3, &spins, sizeof(spins), cudaMemcpyHostToDevice) == cudaSuccess
             ? FFTJ_OK
             : gfail(FFTJ_ERR_CUDA, "group: limit upload failed");
}

int fftj_group_debug_stall(fftj_group g, int op) {
  if (!g) return gfail(FFTJ_ERR_ARG, "null group");
  if (g->mode != FFTJ_GROUP_PERSISTENT) return gfail(FFTJ_ERR_ARG, "stall hook applies to persistent groups");
  if (op < 0 || op >= g->nops || g->h_ops[op].dep < 0) return gfail(FFTJ_ERR_ARG, "op has no dependency to stall");
  const uint32_t need = g->h_ops[g->h_ops[op].dep].ntiles + 1;  // a count no execution reaches
  return cudaMemcpy(&g->d_ops[op].dep_need, &need, sizeof(need), cudaMemcpyHostToDevice) == cudaSuccess
             ? FFTJ_OK
             : gfail(FFTJ_ERR_CUDA, "group: stall upload failed");
}

int fftj_group_destroy(fftj_group g) {
  delete g;
  return FFTJ_OK;
}

}  // extern "C"
