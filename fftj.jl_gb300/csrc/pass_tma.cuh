// Pipelined pass kernel for F32 transforms: the tile columns of a pass of a
// multi-pass transform are contiguous in HBM row by row (MODE 1: first
// passes, columns p; MODE 2: later passes, columns q), so a tile is a box of
// a tensor and arrives in shared memory by TMA tensor copies
// (cp.async.bulk.tensor); a tile of a single-pass transform (MODE 0) is whole
// contiguous transforms, one 1-D bulk copy (cp.async.bulk) each. The copies
// complete on an mbarrier. Each CTA is persistent and double-buffered:
// while it transforms tile i in one buffer, the copy of its next tile lands
// in the other, so HBM reads overlap the in-CTA sub-stages instead of
// waiting for them.
//
// Per tile the work is that of the one-tile-per-CTA recipe kernel
// (pass_fused, the Stockham pass of FFTJ's src/stockham.jl:26-76 with radix
// R): the first sub-stage reads the dense tile the copy left in shared memory
// and writes it back in place in the padded layout, the middle sub-stages run
// in shared memory, and the last one is fused into the HBM store with the
// outer twiddle (store_last).
//
// Every wait is bounded: a copy that has not landed after the plan's wait
// limit sets a status word the host reads (fftj_plan_status), and the CTA
// waits (again bounded) for its copies in flight and returns. The slot
// barriers track only the real copies (the test hook's never-arriving bytes
// sit on a barrier of their own), so that drain observes the copies
// themselves: when it succeeds no copy into this CTA's shared memory is in
// flight as it exits. Only when the copies themselves never land does the
// CTA exit with them outstanding; the host then treats the whole stream's
// results as lost (fftj_plan_status).
#pragma once
#include <cuda.h>

#include "pass_common.cuh"
#include "umma.cuh"

namespace fftj {

__device__ __forceinline__ uint32_t sh_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sh_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sh_addr(bar)), "r"(bytes) : "memory");
}
// true once the barrier's phase of this parity has completed
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(sh_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ uint64_t ns_now() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the phase of the given parity; false after limit_ns nanoseconds.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  if (mbar_test(bar, parity)) return true;
  const uint64_t t0 = ns_now();
  for (;;) {
    for (int i = 0; i < 16; ++i)
      if (mbar_test(bar, parity)) return true;
    if (ns_now() - t0 > limit_ns) return false;
  }
}
// 1-D bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(sh_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(sh_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(sh_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(sh_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load4(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                          int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(sh_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(sh_addr(bar))
      : "memory");
}

// ---------------------------------------------------------------------------
// Precision form on the fifth-generation tensor cores: a radix-16 sub-stage
// as the GEMM Y = X C^T per 128 butterflies (rows), in real form. Operands
// are FP16 hi + lo: each butterfly is scaled by a power of two so that its
// largest component is below 1, split into hi = fp16(x) and lo = fp16((x -
// hi) 2^11) (lo stays a normal number), and likewise the DFT matrix. A row
// of A holds a butterfly's 64 halves [Xr hi | Xi hi | Xr lo | Xi lo]; B has
// 64 rows: rows 0..31 [C hi | 0] give D1 = A_hi C_hi^T, rows 32..63 [C lo |
// C hi] give D2 = A_hi C_lo^T + A_lo C_hi^T (lo * lo dropped), where the 32
// rows of C are the real outputs Yr[n] = Cr Xr - Ci Xi and Yi[n] = Ci Xr +
// Cr Xi, C = w_16^(n j). One accumulator of 64 FP32 columns per block in
// tensor memory, four tcgen05.mma (M = 128, N = 64, K = 16) issued by one
// thread, completion on an mbarrier, read back with tcgen05.ld; Y = (D1 +
// D2 2^-11) unscaled. Same arithmetic as the legacy mma.sync form.
//
// A lives in the tile buffer itself: a butterfly's 16 FP32 inputs are 128
// bytes, as is its row of A, so once every thread holds its inputs in
// registers the tile's bytes become A, and once every MMA is done they take
// the sub-stage's outputs.

// B operand (64 rows x 64 halves, core matrices 128 bytes apart along K,
// 8-row groups 1024 bytes apart) at tcB
template <int DIR>
__device__ __forceinline__ void tc16_b_operand(unsigned char* tcB, int tid, int nthr) {
  for (int e = tid; e < 64 * 32; e += nthr) {
    const int n = e >> 5, k2 = (e & 31) * 2;  // row n, columns k2 and k2 + 1
    float val[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = k2 + h;
      const int row = n & 31, kk = k & 31;     // row of C, column of C
      const int yo = row & 15, xi = kk & 15;  // output and input points
      float sn, cs;
      sincospif((float)((yo * xi) & 15) * 0.125f, &sn, &cs);
      const float cr = cs, ci = DIR * sn;
      // rows 0..15 of C: Yr = Cr Xr - Ci Xi; rows 16..31: Yi = Ci Xr + Cr Xi
      val[h] = row < 16 ? (kk < 16 ? cr : -ci) : (kk < 16 ? ci : cr);
    }
    uint32_t hi, lo;
    split_pair<1>(val[0], val[1], hi, lo);
    // rows 0..31: [C hi | 0]; rows 32..63: [C lo | C hi]
    uint32_t v;
    if (n < 32) v = k2 < 32 ? hi : 0u;
    else v = k2 < 32 ? lo : hi;
    const int off = (n >> 3) * 1024 + (k2 >> 3) * 128 + (n & 7) * 16 + (k2 & 7) * 2;
    *reinterpret_cast<uint32_t*>(tcB + off) = v;
  }
}

// The first sub-stage (radix 16, S = 1) of a pipelined tile on the tensor
// cores: thread tid's butterfly (column c, k) is row tid of the GEMM. Reads
// the dense tile, writes the outputs (twiddled by w_R^(j k) in FP32) to the
// padded layout as the FP32 sub-stage does. False (for every thread) when
// the MMAs did not complete within the wait limit.
template <int DIR, int MODE, int NBC, int R, int Rr, int nthr>
__device__ __forceinline__ bool tc16_first(Cx<float>* buf, const Cx<float>* tw, unsigned char* tcB,
                                           uint64_t* tcbar, uint32_t tmem, uint32_t par, int tid, int b, int kg,
                                           uint64_t limit) {
  using T = float;
  using L = LayC<T, NBC>;
  constexpr int NB = NBC, r0 = 16;
  const int c = MODE == 0 ? tid / Rr : b;
  const int k = MODE == 0 ? tid - c * Rr : kg;
  const Cx<T>* src = MODE == 0 ? buf + c * R + k : buf + k * NB + b;
  constexpr int js = MODE == 0 ? Rr : Rr * NB;
  float xr[16], xi[16];
  float mx = 0.f;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const Cx<T> v = src[j * js];
    xr[j] = v.x;
    xi[j] = v.y;
    mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
  }
  int ex = 0;
  if (mx > 0.f) frexpf(mx, &ex);  // mx < 2^ex
  const float sc = ldexpf(1.f, -ex);
  uint32_t hw[32];  // row tid of A as packed half pairs
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    split_pair<1>(xr[2 * j] * sc, xr[2 * j + 1] * sc, hw[j], hw[16 + j]);
    split_pair<1>(xi[2 * j] * sc, xi[2 * j + 1] * sc, hw[8 + j], hw[24 + j]);
  }
  __syncthreads();  // every input is in registers: the tile's bytes become A
  // row tid: 8 core rows of 16 bytes (row group (tid mod 128) / 8 of block
  // tid / 128, 16 KB per block)
  unsigned char* const tcA = reinterpret_cast<unsigned char*>(buf);
  unsigned char* arow = tcA + (tid >> 7) * 16384 + ((tid & 127) >> 3) * 1024 + (tid & 7) * 16;
#pragma unroll
  for (int kc = 0; kc < 8; ++kc)
    *reinterpret_cast<uint4*>(arow + kc * 128) = make_uint4(hw[4 * kc], hw[4 * kc + 1], hw[4 * kc + 2], hw[4 * kc + 3]);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // A visible to the tensor cores
  __syncthreads();
  if (tid == 0) {
    tc_fence_after();
    constexpr uint32_t kId = umma_idesc_f16(128, 64, 0);
    const uint32_t b0 = sh_addr(tcB);
#pragma unroll 1
    for (int blk = 0; blk < nthr / 128; ++blk) {
      const uint32_t a0 = sh_addr(tcA) + blk * 16384;
      const uint32_t d = tmem + blk * 64;
#pragma unroll
      for (int ks = 0; ks < 4; ++ks)
        umma_f16(d, umma_desc(a0 + ks * 256, 128, 1024), umma_desc(b0 + ks * 256, 128, 1024), kId, ks > 0);
    }
    umma_commit(tcbar);
  }
  const bool ok = mbar_wait(tcbar, par, limit);
  if (__syncthreads_or(!ok)) return false;  // every thread leaves together
  tc_fence_after();
  // row tid = lane 32 (w mod 4) + lane of block w / 4 (warp w)
  const int warp = tid >> 5;
  const uint32_t ta = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(warp >> 2) * 64;
  float d[64];  // D1 (columns 0..31) and D2 (32..63) in one load
  tmem_ld64(ta, d);
  constexpr float kInvLo = 1.f / lo_scale<1>();
  float y[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) y[i] = fmaf(d[32 + i], kInvLo, d[i]);
  tc_fence_before();
  __syncthreads();  // every MMA is done: the outputs may overwrite A
  const float us = ldexpf(1.f, ex);
  constexpr bool kLay = L::exact(r0);
  const int a = r0 * k * NB + c;
  const int base = kLay ? L::row(r0 * k) + L::col(c) : pidx<T>(a);
  buf[base] = mk<T>(y[0] * us, y[16] * us);
#pragma unroll
  for (int j = 1; j < r0; ++j) {
    Cx<T> w = mk<T>(y[j] * us, y[16 + j] * us);
    if (k != 0) w = cmul(w, tw[j * k]);
    buf[kLay ? base + L::step(j) : pidx<T>(a + j * NB)] = w;
  }
  __syncthreads();
  return true;
}

// MODE 0: tile = NB whole contiguous transforms (batch entries), one 1-D
// bulk copy per entry; MODE 1: tile = P consecutive columns p (Q == 1, one
// batch entry), tensor (p, j, batch); MODE 2: tile = Q consecutive columns q
// (P == 1, one batch entry), tensor (q, p, j, batch). NBC = the tile's
// column count. The pass's inner twiddles w_R^t are staged in shared memory
// once per CTA (up to R = 4096, 32 KB: the radix-4096 single pass then runs
// two CTAs per SM, measured faster than three reading them through L1).
template <int R>
__host__ __device__ constexpr bool tma_stages_twiddles() { return R <= 4096; }

// TC = 1: the precision form (FP16 hi + lo operands): the first sub-stage,
// radix 16 with one butterfly per thread, runs on the tensor cores as one
// tcgen05 GEMM per 128 butterflies (tc16_first below).
template <int DIR, int MODE, int NBC, int TC, int... Rs>
__device__ __forceinline__ void pass_tma(const PassParams& pp, const CUtensorMap* map, const Cx<float>* in,
                                         Cx<float>* __restrict__ out, unsigned* status) {
  using T = float;
  using Rec = Recipe<Rs...>;
  using L = LayC<T, NBC>;
  constexpr int R = Rec::R, TF = Rec::Tf, NS = Rec::n;
  constexpr int rad[] = {Rs...};
  constexpr int r0 = rad[0];
  constexpr int Rr = R / r0;
  constexpr int IPT = (Rr + TF - 1) / TF;
  constexpr int NB = NBC;
  constexpr int nthr = NBC * TF;
  constexpr uint32_t kTx = (uint32_t)(NB * R * sizeof(Cx<T>));
  static_assert(NS >= 2, "the first and last sub-stages are separate");
  static_assert(MODE != 0 || Rr % TF == 0, "single-pass tiles: whole butterfly rounds per thread");
  constexpr bool kTc = TC != 0;
  static_assert(!kTc || (r0 == 16 && IPT == 1 && Rr == TF && nthr % 128 == 0),
                "tensor-core first sub-stage: radix 16, one butterfly per thread, whole 128-thread blocks");
  constexpr uint32_t kTcCols = (uint32_t)(nthr / 128) * 64;  // D1 and D2, 32 columns each, per 128 rows
  // box copies land 16-byte aligned: dynamic shared memory starts 16-byte
  // aligned and buffers are multiples of 128 bytes
  extern __shared__ __align__(16) unsigned char tma_smem[];
  Cx<T>* const sbase = reinterpret_cast<Cx<T>*>(tma_smem);
  const int bufE = pp.tma_buf;  // elements per buffer, a multiple of 16 (128 bytes)
  constexpr bool kStageTw = tma_stages_twiddles<R>();
  Cx<T>* const twS = sbase + 2 * bufE;
  uint64_t* const bar = reinterpret_cast<uint64_t*>(twS + (kStageTw ? R : 0));
  const Cx<T>* const tw = kStageTw ? twS : reinterpret_cast<const Cx<T>*>(pp.twR);
  const int tid = threadIdx.x;
  const int kg = tid / NB;
  const int b = tid - kg * NB;
  // tensor-core B operand after the kernel's own shared memory (A lives in
  // the tile buffer)
  unsigned char* const tcB =
      tma_smem + tc_smem_offset((size_t)(2 * bufE + (kStageTw ? R : 0)) * sizeof(Cx<T>) + 3 * sizeof(uint64_t));
  uint64_t* const tcbar = reinterpret_cast<uint64_t*>(tcB + 8192);
  uint32_t* const tmem_slot = reinterpret_cast<uint32_t*>(tcbar + 1);
  const uint32_t ntiles = pp.tiles_q * pp.tiles_p * pp.tiles_b;
  const int rows = pp.tma_rows;
  const uint64_t limit = pp.tma_wait_ns;
  if constexpr (kStageTw) {
    const Cx<T>* twG = reinterpret_cast<const Cx<T>*>(pp.twR);
    for (int t = tid; t < R; t += nthr) twS[t] = __ldg(twG + t);
  }
  // bar[0], bar[1]: the two tile slots (real copies only); bar[2]: the test
  // hook (fftj_plan_debug_stall) -- armed once with bytes that never arrive,
  // and waited on after each slot's barrier, so every tile wait times out
  // while the slot barriers still see their copies land
  const uint32_t extra_tx = (uint32_t)pp.tma_extra_tx;
  if constexpr (kTc) tc16_b_operand<DIR>(tcB, tid, nthr);
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_init(bar + 1, 1);
    mbar_init(bar + 2, 1);
    if constexpr (kTc) mbar_init(tcbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (extra_tx) mbar_arrive_expect_tx(bar + 2, extra_tx);
  }
  if constexpr (kTc) {
    if (tid < 32) tmem_alloc(tmem_slot, kTcCols);
    tc_fence_before();
  }
  __syncthreads();
  uint32_t tmem = 0, tc_par = 0;
  if constexpr (kTc) {
    tc_fence_after();
    tmem = *tmem_slot;
  }
  // tensor memory back before any exit (every thread; warp 0 allocated it)
  auto tc_release = [&]() {
    if constexpr (kTc) {
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (tid < 32) tmem_dealloc(tmem, kTcCols);
    }
  };
  // one thread arms the slot's barrier with the tile's bytes and issues the
  // tile's box copies (R / rows boxes of NB x rows elements)
  auto issue = [&](uint32_t tile, int slot) {
    const uint32_t t1 = pp.ftq.div(tile);
    const uint32_t tq = tile - t1 * pp.tiles_q;
    const uint32_t tb = pp.ftp.div(t1);
    const uint32_t tp = t1 - tb * pp.tiles_p;
    Cx<T>* dst = sbase + slot * bufE;
    if constexpr (MODE == 0) {
      // the tile's batch entries that exist, each R contiguous elements
      const int64_t b0 = (int64_t)tb * NB;
      const int nv = (int)min((int64_t)NB, pp.nbatch - b0);
      mbar_arrive_expect_tx(bar + slot, (uint32_t)(nv * R * sizeof(Cx<T>)));
      for (int c = 0; c < nv; ++c)
        bulk_load(dst + c * R, in + (b0 + c) * pp.in_bstride, (uint32_t)(R * sizeof(Cx<T>)), bar + slot);
    } else {
      mbar_arrive_expect_tx(bar + slot, kTx);
      for (int j0 = 0; j0 < R; j0 += rows) {
        if constexpr (MODE == 1)
          tma_load3(dst + j0 * NB, map, bar + slot, (int)(tp * (uint32_t)pp.P), j0, (int)tb);
        else
          tma_load4(dst + j0 * NB, map, bar + slot, (int)(tq * (uint32_t)pp.Q), (int)tp, j0, (int)tb);
      }
    }
  };
  if (tid == 0 && blockIdx.x < ntiles) issue(blockIdx.x, 0);
  uint32_t it = 0;
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int slot = (int)(it & 1);
    Cx<T>* const buf = sbase + slot * bufE;
    const uint32_t nxt = tile + gridDim.x;
    if (tid == 0 && nxt < ntiles) {
      // the other buffer was last read (generic proxy) before the barrier
      // that ended the previous tile; order those reads before the copy
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(nxt, slot ^ 1);
    }
    const bool ok = mbar_wait(bar + slot, (it >> 1) & 1, limit) && (extra_tx == 0 || mbar_wait(bar + 2, 0, limit));
    if (__syncthreads_or(!ok)) {
      // drain: wait (bounded) for this tile's copies and the next tile's,
      // on the slot barriers that count only real copy bytes
      if (tid == 0) {
        atomicOr(status, 1u);
        bool drained = mbar_wait(bar + slot, (it >> 1) & 1, limit);
        if (nxt < ntiles) drained = mbar_wait(bar + (slot ^ 1), ((it + 1) >> 1) & 1, limit) && drained;
        if (!drained) atomicOr(status, 2u);  // copies still in flight at exit
      }
      __syncthreads();
      tc_release();
      return;
    }
    const uint32_t t1 = pp.ftq.div(tile);
    const uint32_t tq = tile - t1 * pp.tiles_q;
    const uint32_t tb = pp.ftp.div(t1);
    const uint32_t tp = t1 - tb * pp.tiles_p;
    const int64_t q0 = (int64_t)tq * pp.Q, p0 = (int64_t)tp * pp.P, b0 = (int64_t)tb * (MODE == 0 ? NB : 1);
    const int ql = MODE == 2 ? b : 0;
    const int64_t pcol = MODE == 1 ? p0 + b : p0;
    const bool colok = b0 < pp.nbatch && q0 + ql < pp.s;

    // ---- first sub-stage (radix r0, S = 1) from the dense tile, written
    // back in place in the padded layout
    // butterfly (column c, k): MODE 0 takes k fastest across lanes (entries
    // are rows [c][j] of the dense tile), modes 1 and 2 the column (rows
    // [j][c]); both read consecutive addresses across a warp
    if constexpr (kTc) {
      const bool tok = tc16_first<DIR, MODE, NBC, R, Rr, nthr>(buf, tw, tcB, tcbar, tmem, tc_par, tid, b, kg, limit);
      tc_par ^= 1u;
      if (!tok) {  // uniform: decided by a block-wide vote
        // the MMAs did not complete: record it, drain the next tile's copy
        // (bounded) and leave
        if (tid == 0) {
          atomicOr(status, 1u);
          if (nxt < ntiles && !mbar_wait(bar + (slot ^ 1), ((it + 1) >> 1) & 1, limit)) atomicOr(status, 2u);
        }
        __syncthreads();
        tc_release();
        return;
      }
    } else {
    Cx<T> v[IPT][r0];
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      const int u = tid + i * nthr;
      const int c = MODE == 0 ? u / Rr : b;
      const int k = MODE == 0 ? u - c * Rr : kg + i * TF;
      if (MODE == 0 || (i + 1) * TF <= Rr || k < Rr) {
        const Cx<T>* src = MODE == 0 ? buf + c * R + k : buf + k * NB + b;
        constexpr int js = MODE == 0 ? Rr : Rr * NB;
#pragma unroll
        for (int j = 0; j < r0; ++j) v[i][j] = src[j * js];
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < IPT; ++i) {
      const int u = tid + i * nthr;
      const int c = MODE == 0 ? u / Rr : b;
      const int k = MODE == 0 ? u - c * Rr : kg + i * TF;
      if (MODE == 0 || (i + 1) * TF <= Rr || k < Rr) {
        Dft<T, DIR, r0>::run(v[i]);
        constexpr bool kLay = L::exact(r0);
        const int a = r0 * k * NB + c;
        const int base = kLay ? L::row(r0 * k) + L::col(c) : pidx<T>(a);
        buf[base] = v[i][0];
#pragma unroll
        for (int j = 1; j < r0; ++j) {
          Cx<T> w = v[i][j];
          if (k != 0) w = cmul(w, tw[j * k]);
          buf[kLay ? base + L::step(j) : pidx<T>(a + j * NB)] = w;
        }
      }
    }
    __syncthreads();
    }
    if constexpr (NS > 2) run_mid_ct<T, DIR, TF, R, r0, 1, NBC, Rs...>(buf, b, kg, NB, tw);
    store_last<T, DIR, MODE, NBC, Rs...>(pp, out, buf, tid, nthr, kg, b, b0, p0, q0, ql, b0, pcol, colok);
    __syncthreads();  // the buffer is free for the copy after next
  }
  tc_release();
}

template <int DIR, int MODE, int NBC, class Rec, int TC = 0>
struct TmaLaunch;
template <int DIR, int MODE, int NBC, int TC, int... Rs>
struct TmaLaunch<DIR, MODE, NBC, Recipe<Rs...>, TC> {
  __device__ __forceinline__ static void run(const PassParams& pp, const CUtensorMap* map, const Cx<float>* in,
                                             Cx<float>* out, unsigned* status) {
    pass_tma<DIR, MODE, NBC, TC, Rs...>(pp, map, in, out, status);
  }
};

}  // namespace fftj
