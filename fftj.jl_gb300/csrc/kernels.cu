// sm_103a kernels of the FFTJ transform path.
//
// The hot kernel is one Stockham "super-radix" pass (k_pass): each CTA loads a
// tile of butterfly columns (batch x p x q) from HBM with coalesced accesses,
// runs the pass's R-point DFTs as a chain of register radix sub-stages
// (2/3/4/5/7/8/11/13/16) ping-ponging through shared memory, applies the
// pass's outer twiddle w_ncur^(p*j) and writes the tile back. A 1-D transform
// of length N = R1*R2*...*Rk is k such passes (the Stockham stage of
// FFTJ's src/stockham.jl:26-130 with radix R_i instead of 4/8), i.e. the
// four-step/six-step family (src/fourstep.jl) with the transposes folded into
// the Stockham index maps. N-d passes are the same kernel with the inner
// dims folded into the stride s (src/ndplan.jl:1-5: "effective stride s*Bi").
#include <cuda_runtime.h>

#include "elementwise.cuh"
#include "pass_common.cuh"

namespace fftj {

template <typename T, int DIR, int LOADOP>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256, 2)
    k_pass(const __grid_constant__ PassParams pp, const void* __restrict__ in, Cx<Hs<T>>* __restrict__ out) {
  pass_body<T, DIR, LOADOP, RuntimeRecipe>(pp, in, out);
}

template <typename T>
__global__ void k_interp(const __grid_constant__ InterpParams ip, const Cx<T>* __restrict__ g,
                         Cx<T>* __restrict__ y) {
  interp_at<T, false>(ip, g, y, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <typename T, int B>
__global__ void k_hvdh_solve(const __grid_constant__ SolveParams sp, const Cx<T>* __restrict__ g,
                             Cx<T>* __restrict__ y) {
  solve_at<T, B, false>(sp, g, y, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// the same solve with its factors rebuilt per call (a kernel of its own, so
// that the tabulated solve keeps its registers)
template <typename T, int B>
__global__ void k_hvdh_solve_fly(const __grid_constant__ SolveParams sp, const Cx<T>* __restrict__ g,
                                 Cx<T>* __restrict__ y) {
  solve_fly_at<T, B, false>(sp, g, y, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <typename T>
__global__ void k_real_post(const RealPostParams rp, const Cx<T>* __restrict__ z, Cx<T>* __restrict__ y) {
  real_post_at<T, false>(rp, z, y, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <typename T>
__global__ void k_copy(const CopyParams cp, const void* __restrict__ in, void* __restrict__ out) {
  copy_at<T, false>(cp, in, out, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------
template <typename T>
using PassFn = void (*)(const PassParams, const void*, Cx<Hs<T>>*);

template <typename T>
static PassFn<T> pass_fn(int dir, int load_op) {
  if (dir < 0) {
    switch (load_op) {
      case LOAD_DECONV: return k_pass<T, -1, LOAD_DECONV>;
      case LOAD_C2R_PRE: return k_pass<T, -1, LOAD_C2R_PRE>;
      case LOAD_REAL: return k_pass<T, -1, LOAD_REAL>;
      case LOAD_SPREAD: return k_pass<T, -1, LOAD_SPREAD>;
      default: return k_pass<T, -1, LOAD_PLAIN>;
    }
  }
  switch (load_op) {
    case LOAD_DECONV: return k_pass<T, 1, LOAD_DECONV>;
    case LOAD_C2R_PRE: return k_pass<T, 1, LOAD_C2R_PRE>;
    case LOAD_REAL: return k_pass<T, 1, LOAD_REAL>;
    case LOAD_SPREAD: return k_pass<T, 1, LOAD_SPREAD>;
    default: return k_pass<T, 1, LOAD_PLAIN>;
  }
}

// The generic kernel of a pass: ComplexF64 passes compute in block fixed
// point unless the plan asked for FP64 butterflies.
template <typename T>
static const void* generic_pass(const PassParams& pp, int dir) {
  if constexpr (sizeof(T) == 8) {
    if (pp.fx) return (const void*)pass_fn<Fx>(dir, pp.load_op);
  }
  return (const void*)pass_fn<T>(dir, pp.load_op);
}
// dynamic shared memory of a pass: the tile (two tile buffers for the
// generic kernel, which ping-pongs between them), staged twiddles and (block
// fixed point) the column exponents
static size_t pass_smem(const PassParams& pp, size_t esz, bool generic) {
  return (size_t)((generic ? 2 : 1) * pp.smem_elems + pp.smem_tw_elems) * esz + (size_t)pp.fx_cols * sizeof(int);
}

// Opt a pass kernel into the device's largest dynamic shared memory. The
// attribute belongs to the kernel function (shared by every plan), so it is
// never set below the maximum any plan may need.
template <typename T>
cudaError_t prepare_pass(const PassParams& pp, int dir, const void* fn) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const void* f = fn ? fn : generic_pass<T>(pp, dir);
  // the dynamic limit is what the device allows per block minus the
  // kernel's own static shared memory
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, f);
  if (e != cudaSuccess) return e;
  const int maxdyn = optin - (int)fa.sharedSizeBytes;
  const size_t need = pass_smem(pp, sizeof(Cx<T>), fn == nullptr);
  if (maxdyn <= 0 || need > (size_t)maxdyn) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, maxdyn);
}

template <typename T>
cudaError_t launch_pass(const PassParams& pp, int dir, const void* fn, const void* in, void* out,
                        cudaStream_t st) {
  const size_t smem = pass_smem(pp, sizeof(Cx<T>), fn == nullptr);
  const uint32_t grid = pp.tiles_q * pp.tiles_p * pp.tiles_b;
  const void* f = fn ? fn : generic_pass<T>(pp, dir);
  void* args[3] = {const_cast<PassParams*>(&pp), const_cast<void**>(&in), &out};
  return cudaLaunchKernel(f, dim3(grid), dim3(pp.threads), args, smem, st);
}

template <typename T>
cudaError_t launch_interp(const InterpParams& ip, const void* g, void* y, cudaStream_t st) {
  const int64_t total = ip.n * ip.nbatch * (ip.inner > 1 ? ip.inner : 1);
  const int th = 256;
  k_interp<T><<<(unsigned)((total + th - 1) / th), th, 0, st>>>(ip, reinterpret_cast<const Cx<T>*>(g),
                                                                reinterpret_cast<Cx<T>*>(y));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_real_post(const RealPostParams& rp, const void* z, void* y, cudaStream_t st) {
  const int64_t total = (rp.h / 2 + 1) * rp.nbatch;  // one thread per pair (k, h - k)
  const int th = 256;
  k_real_post<T><<<(unsigned)((total + th - 1) / th), th, 0, st>>>(rp, reinterpret_cast<const Cx<T>*>(z),
                                                                   reinterpret_cast<Cx<T>*>(y));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_copy(const CopyParams& cp, const void* in, void* out, cudaStream_t st) {
  const int64_t total = cp.n * cp.nbatch;
  const int th = 256;
  k_copy<T><<<(unsigned)((total + th - 1) / th), th, 0, st>>>(cp, in, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_solve(const SolveParams& sp, const void* g, void* y, cudaStream_t st) {
  const int64_t total = sp.nbatch * sp.nchunk;
  // one warp per CTA: the solve is FP64-pipe bound and has few threads
  // (batch x chunks), so small CTAs spread it over every SM
  const int th = 32;
  const unsigned grid = (unsigned)((total + th - 1) / th);
  auto gg = reinterpret_cast<const Cx<T>*>(g);
  auto yy = reinterpret_cast<Cx<T>*>(y);
  if (sp.fly) {
    switch (sp.B) {
      case 1: k_hvdh_solve_fly<T, 1><<<grid, th, 0, st>>>(sp, gg, yy); break;
      case 2: k_hvdh_solve_fly<T, 2><<<grid, th, 0, st>>>(sp, gg, yy); break;
      case 3: k_hvdh_solve_fly<T, 3><<<grid, th, 0, st>>>(sp, gg, yy); break;
      default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
  }
  switch (sp.B) {
    case 1: k_hvdh_solve<T, 1><<<grid, th, 0, st>>>(sp, gg, yy); break;
    case 2: k_hvdh_solve<T, 2><<<grid, th, 0, st>>>(sp, gg, yy); break;
    case 3: k_hvdh_solve<T, 3><<<grid, th, 0, st>>>(sp, gg, yy); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template cudaError_t launch_solve<float>(const SolveParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_solve<double>(const SolveParams&, const void*, void*, cudaStream_t);
template cudaError_t prepare_pass<float>(const PassParams&, int, const void*);
template cudaError_t prepare_pass<double>(const PassParams&, int, const void*);
template cudaError_t launch_pass<float>(const PassParams&, int, const void*, const void*, void*, cudaStream_t);
template cudaError_t launch_pass<double>(const PassParams&, int, const void*, const void*, void*, cudaStream_t);
template cudaError_t launch_interp<float>(const InterpParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_interp<double>(const InterpParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_real_post<float>(const RealPostParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_real_post<double>(const RealPostParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_copy<float>(const CopyParams&, const void*, void*, cudaStream_t);
template cudaError_t launch_copy<double>(const CopyParams&, const void*, void*, cudaStream_t);

}  // namespace fftj
