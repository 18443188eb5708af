// Host-side plan representation shared by the planner (planner.cpp) and
// the group executor (group.cu): a plan is a list of ops (passes and
// elementwise kernels) wired between the caller's in/out buffers and two
// plan-owned workspaces.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <vector>

#include "../../include/fftj.h"
#include "fftj_internal.h"

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

enum OpKind { OP_PASS = 0, OP_INTERP = 1, OP_RPOST = 2, OP_COPY = 3, OP_SOLVE = 4 };
enum BufId { B_IN = 0, B_OUT = 1, B_W0 = 2, B_W1 = 3 };

struct Op {
  OpKind kind;
  int src, dst;
  int dir = -1;
  const void* kfn = nullptr;  // recipe kernel for OP_PASS (nullptr: generic)
  fftj::PassParams pp;
  fftj::InterpParams ip;
  fftj::RealPostParams rp;
  fftj::CopyParams cp;
  fftj::SolveParams sv;
  size_t dst_bytes = 0;  // bytes written (for workspace sizing)
  // pipelined tensor-copy kernel of an F32 pass (nullptr: none); its tensor
  // map is encoded for the source address tmap_src on first use
  const void* kfn_tma = nullptr;
  int tma_mode = 0;  // 1: columns p (first pass), 2: columns q (later pass)
  int tma_grid = 0;  // CTAs resident at once (the persistent grid)
  CUtensorMap tmap;
  const void* tmap_src = nullptr;
};

struct fftj_plan_s {
  int dtype = 0;
  int kind = 0;  // 0 c2c, 1 r2c, 2 c2r
  int route = FFTJ_ROUTE_DIRECT;
  std::vector<int64_t> dims;
  int64_t n = 1, batch = 1;
  int64_t resample_m = 0, resample_w = 0;
  std::vector<Op> ops;
  std::vector<DevBuf> tables;
  DevBuf ws[2];
  size_t table_bytes = 0;
  bool inplace_safe = false;
  bool dry = false;
  int npasses = 0;
  std::vector<int> pass_R;
  int plain_loads = 0;            // opts.plain_loads
  unsigned* d_status = nullptr;   // pipelined kernels' wait status (0: every wait ended)
  ~fftj_plan_s() {
    if (d_status) cudaFree(d_status);
    for (auto& t : tables)
      if (t.p && t.bytes) cudaFree(t.p);
    for (auto& w : ws)
      if (w.p) cudaFree(w.p);
  }
};
