// Pipelined pass kernels of the precision form (F32, FP16 hi + lo): the
// pass_tma kernels of the recipes whose first sub-stage is radix 16 with
// one butterfly per thread, that sub-stage on the tensor cores (tcgen05).
// The tensor-core operands take shared memory beside the tile buffers, so
// these run two CTAs of 256 threads per SM (one of 512).
#include "pass_tma.cuh"

namespace fftj {

template <int DIR, int MODE, int NBC, class Rec>
__global__ void __launch_bounds__(NBC * Rec::Tf, NBC * Rec::Tf <= 256 ? 2 : 1)
    k_tma_tc(const __grid_constant__ PassParams pp, const __grid_constant__ CUtensorMap map,
             const Cx<float>* __restrict__ in, Cx<float>* __restrict__ out, unsigned* status) {
  TmaLaunch<DIR, MODE, NBC, Rec, 1>::run(pp, &map, in, out, status);
}

#define TC_(DIR, MODE, NB, ...)                                                                         \
  {0, DIR, LOAD_PLAIN, MODE, {__VA_ARGS__}, Recipe<__VA_ARGS__>::Tf, NB,                                 \
   (const void*)k_tma_tc<DIR, MODE, NB, Recipe<__VA_ARGS__>>, 1},
#define TCT_(NB, ...)                                                                                   \
  TC_(-1, 1, NB, __VA_ARGS__) TC_(-1, 2, NB, __VA_ARGS__) TC_(1, 1, NB, __VA_ARGS__) TC_(1, 2, NB, __VA_ARGS__)
#define TC0_(NB, ...) TC_(-1, 0, NB, __VA_ARGS__) TC_(1, 0, NB, __VA_ARGS__)

static const RecipeEntry kTmaTc[] = {
    // multi-pass transforms: radix 128, 256 and 1024 passes (4096- and
    // 8192-element tiles)
    TCT_(32, 16, 8) TCT_(16, 16, 16) TCT_(8, 16, 8, 8) TCT_(64, 16, 8) TCT_(32, 16, 16)
    // single-pass transforms of three sub-stages (4096- and 8192-element tiles)
    TC0_(1, 16, 16, 16) TC0_(2, 16, 16, 8) TC0_(4, 16, 8, 8) TC0_(2, 16, 16, 16) TC0_(4, 16, 16, 8)
    TC0_(8, 16, 8, 8)
};

const RecipeEntry* tma_tc_table(int* count) {
  *count = (int)(sizeof(kTmaTc) / sizeof(kTmaTc[0]));
  return kTmaTc;
}

}  // namespace fftj
