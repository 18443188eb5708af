// Pipelined tensor-copy pass kernels (pass_tma.cuh), F32, for the power-of-
// two passes of multi-pass transforms and the three-sub-stage single passes
// at the planner's default tiles, with the host helpers that size and launch
// them.
#include <algorithm>

#include "pass_tma.cuh"

namespace fftj {

// 256-thread tiles keep 3 CTAs per SM (registers <= 85); the 512-thread
// radix-1024 tile runs one
template <int DIR, int MODE, int NBC, class Rec>
__global__ void __launch_bounds__(NBC * Rec::Tf, NBC * Rec::Tf <= 256 ? 3 : 1)
    k_tma(const __grid_constant__ PassParams pp, const __grid_constant__ CUtensorMap map,
          const Cx<float>* __restrict__ in, Cx<float>* __restrict__ out, unsigned* status) {
  TmaLaunch<DIR, MODE, NBC, Rec>::run(pp, &map, in, out, status);
}

#define T_(DIR, MODE, NB, ...) \
  {0, DIR, LOAD_PLAIN, MODE, {__VA_ARGS__}, Recipe<__VA_ARGS__>::Tf, NB, (const void*)k_tma<DIR, MODE, NB, Recipe<__VA_ARGS__>>},
#define TT_(NB, ...)                                                                                \
  T_(-1, 1, NB, __VA_ARGS__) T_(-1, 2, NB, __VA_ARGS__) T_(1, 1, NB, __VA_ARGS__) T_(1, 2, NB, __VA_ARGS__)
#define T0_(NB, ...) T_(-1, 0, NB, __VA_ARGS__) T_(1, 0, NB, __VA_ARGS__)

static const RecipeEntry kTma[] = {
    // passes of multi-pass transforms (first: mode 1, later: mode 2)
    TT_(128, 8, 4) TT_(64, 8, 8) TT_(32, 16, 8) TT_(16, 16, 16) TT_(8, 8, 8, 8) TT_(8, 16, 8, 8)
    // single-pass transforms of three sub-stages at 4096-element tiles
    T0_(1, 16, 16, 16) T0_(2, 16, 16, 8) T0_(4, 16, 8, 8) T0_(8, 8, 8, 8)
};

const RecipeEntry* tma_table(int dir, int* count) {
  (void)dir;
  *count = (int)(sizeof(kTma) / sizeof(kTma[0]));
  return kTma;
}

size_t tma_smem_bytes(const PassParams& pp) {
  const int tw = pp.R <= 4096 ? pp.R : 0;  // tma_stages_twiddles
  const size_t own = (size_t)(2 * pp.tma_buf + tw) * sizeof(Cx<float>) + 3 * sizeof(uint64_t);  // 3 mbarriers
  // the precision form's tensor-core operands follow (umma.cuh)
  return pp.tc == 1 ? tc_smem_offset(own) + tc_smem_bytes(pp.threads) : own;
}

// Opts the kernel into the shared memory it needs and returns how many CTAs
// of it fit the device at once (the persistent grid), 0 if none.
int tma_prepare(const void* fn, const PassParams& pp) {
  int dev = 0, optin = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  const size_t smem = tma_smem_bytes(pp);
  if (smem > (size_t)optin) return 0;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess) return 0;
  if (pp.tc == 1) {
    // Kernels with tensor-memory instructions: the runtime's occupancy query
    // answers 1 (or 0) CTA per SM for them whatever their resources (checked
    // on a GB300 with the same kernel with and without tcgen05), so the
    // residency comes from the kernel's own limits: shared memory,
    // registers, threads and its tensor-memory columns (512 per SM).
    int smsm = 0, resv = 0;
    cudaFuncAttributes fa;
    if (cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, fn) != cudaSuccess)
      return 0;
    const int warps = (pp.threads + 31) / 32;
    const int regs_warp = (fa.numRegs * 32 + 255) / 256 * 256;
    const int by_smem = smsm / (int)(smem + fa.sharedSizeBytes + resv);
    const int by_regs = 65536 / std::max(1, warps * regs_warp);
    const int by_threads = 2048 / std::max(1, pp.threads);
    const int by_tmem = 512 / std::max(64, (pp.threads / 128) * 64);
    // (two 256-thread CTAs per SM run the radix-4096 rows of 4096^2 in
    // 0.079 ms where the query's one took 0.099 ms)
    per_sm = std::min(std::min(by_smem, by_regs), std::min(by_threads, by_tmem));
    return per_sm > 0 ? per_sm * nsm : 0;
  }
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, pp.threads, smem) != cudaSuccess) return 0;
  return per_sm * nsm;
}

cudaError_t tma_launch(const void* fn, const PassParams& pp, const CUtensorMap& map, const void* in, void* out,
                       unsigned* status, int grid, cudaStream_t st) {
  const uint32_t ntiles = pp.tiles_q * pp.tiles_p * pp.tiles_b;
  const unsigned g = (unsigned)std::min<uint64_t>((uint64_t)grid, ntiles);
  void* args[5] = {const_cast<PassParams*>(&pp), const_cast<CUtensorMap*>(&map), &in, &out, &status};
  return cudaLaunchKernel(fn, dim3(g), dim3(pp.threads), args, tma_smem_bytes(pp), st);
}

}  // namespace fftj
