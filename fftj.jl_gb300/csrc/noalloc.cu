// Allocation-free transform entry point (no counterpart in the reference).
//
// Some callers cannot allocate device memory when they need a transform:
// real-time pipelines that forbid allocation once running (an allocation can
// block on the driver for an unbounded time), and hosts that own every byte
// of device memory through their own pool and have no way to hand a plan its
// workspace. Plans (fftj_plan_c2c) allocate their
// twiddle tables and workspace when they are created; this entry point
// allocates nothing. Its scratch -- the intermediate of a two-pass transform
// and the twiddle tables, which it regenerates on the device on every call --
// is a file-scope static __device__ array of kNoAllocBytes (64 MiB) that every
// GPU which loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/fftj.h"
#include "fftj_internal.h"
#include "fx64.cuh"

namespace fftj {

constexpr size_t kNoAllocBytes = size_t(64) << 20;      // whole scratch array
constexpr size_t kNoAllocTableBytes = size_t(1) << 20;  // first MiB: twiddle tables
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device addresses of g_noalloc_scratch, one per device, looked up on the
// first call made with that device current and kept for the life of the
// process (a device reset after that first call is not supported). In host
// code the symbol's name is a host-side stand-in, not a device address.
static void* g_scratch_addr[kMaxDevices];
static std::mutex g_scratch_mu;

template <typename T>
struct Cplx;
template <>
struct Cplx<float> { using t = float2; };
template <>
struct Cplx<double> { using t = double2; };

// dst[i] = exp(dir * 2 pi i (i*stride mod n) / n), generated in FP64 with an
// exact integer reduction of the exponent; as Q61 integers (the twiddles of
// block fixed-point ComplexF64 passes) when q61 is set.
template <typename T>
__global__ void k_fill_omega(typename Cplx<T>::t* dst, int64_t count, int64_t stride, int64_t n, int dir,
                             int q61) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int64_t r = (i * stride) % n;
  double s, c;
  sincospi(2.0 * (double)r / (double)n, &s, &c);
  if (sizeof(T) == 8 && q61) {
    longlong2 q;
    q.x = fx_q61(c);
    q.y = fx_q61(dir * s);
    reinterpret_cast<longlong2*>(dst)[i] = q;
    return;
  }
  typename Cplx<T>::t w;
  w.x = (T)c;
  w.y = (T)(dir * s);
  dst[i] = w;
}

static cudaError_t scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

template <typename T>
static int run_noalloc(int64_t n, int64_t batch, int dir, double scale, const void* d_in, void* d_out,
                       cudaStream_t st) {
  using C = typename Cplx<T>::t;
  const bool f64 = sizeof(T) == 8;
  int64_t Rs[2];
  const int npass = pass_radices(n, f64, false, Rs, 2);
  if (npass < 1 || npass > 2) {
    set_error("fftj_execute_noalloc_c2c: n must be 13-smooth and run in one or two passes (n <= 2^20 F32, 2^18 F64)");
    return FFTJ_ERR_UNSUPPORTED;
  }
  const size_t data_bytes = (size_t)n * (size_t)batch * sizeof(C);
  if (npass == 2 && data_bytes > kNoAllocBytes - kNoAllocTableBytes) {
    set_error("fftj_execute_noalloc_c2c: batch * n exceeds the 63 MiB scratch array");
    return FFTJ_ERR_ARG;
  }
  void* base = nullptr;
  cudaError_t e = scratch_address(&base);
  if (e != cudaSuccess) {
    set_error("fftj_execute_noalloc_c2c: cudaGetSymbolAddress failed");
    return FFTJ_ERR_CUDA;
  }
  unsigned char* tab = static_cast<unsigned char*>(base);
  unsigned char* data = tab + kNoAllocTableBytes;
  size_t cursor = 0;
  auto table = [&](int64_t count, int64_t stride, int64_t modn, int q61) -> C* {
    C* p = reinterpret_cast<C*>(tab + cursor);
    cursor += ((size_t)count * sizeof(C) + 255) / 256 * 256;
    if (cursor > kNoAllocTableBytes) return nullptr;
    const int th = 256;
    k_fill_omega<T><<<(unsigned)((count + th - 1) / th), th, 0, st>>>(p, count, stride, modn, dir, q61);
    if (cudaGetLastError() != cudaSuccess) return nullptr;  // this launch's own error
    return p;
  };

  PassParams pp[2];
  int64_t s1 = 1, ncur = n;
  for (int i = 0; i < npass; ++i) {
    const int64_t R = Rs[i];
    PassParams& p = pp[i];
    p = PassParams();
    const int64_t m = ncur / R;
    int rc = pass_geometry(p, f64, R, m, s1, ncur, batch, n, n);
    if (rc) return rc;
    p.twR = table(R, 1, R, p.fx);
    if (m > 1) {
      // two-level outer twiddles: O(sqrt(n)) entries fit the table region
      int sh = 0;
      while (((int64_t)1 << (2 * sh)) < ncur) sh++;
      const int64_t K = (int64_t)1 << sh;
      p.tw_mode = 2;
      p.tw_shift = sh;
      p.tw_hi = table((ncur + K - 1) / K, K, ncur, p.fx);
      p.tw_lo = table(K, 1, ncur, p.fx);
      if (!p.tw_hi || !p.tw_lo) {
        set_error("fftj_execute_noalloc_c2c: twiddle tables exceed the table region, or their generation "
                  "failed to launch");
        return FFTJ_ERR_UNSUPPORTED;
      }
    }
    if (!p.twR) {
      set_error("fftj_execute_noalloc_c2c: twiddle tables exceed the table region, or their generation "
                "failed to launch");
      return FFTJ_ERR_UNSUPPORTED;
    }
    p.scale = (i + 1 == npass) ? scale : 1.0;
    p.load_op = LOAD_PLAIN;
    s1 *= R;
    ncur /= R;
  }
  const void* src = d_in;
  for (int i = 0; i < npass; ++i) {
    void* dst = (i + 1 == npass) ? d_out : (void*)data;
    const void* fn = pick_pass_kernel(f64, dir, pp[i]);
    pp[i].smem_tw_elems = stage_inner_twiddles(pp[i], fn != nullptr) ? pp[i].R : 0;
    if (prepare_pass<T>(pp[i], dir, fn) != cudaSuccess ||
        launch_pass<T>(pp[i], dir, fn, src, dst, st) != cudaSuccess) {
      set_error("fftj_execute_noalloc_c2c: pass launch failed");
      return FFTJ_ERR_CUDA;
    }
    src = dst;
  }
  set_error("");
  return FFTJ_OK;
}

}  // namespace fftj

extern "C" int fftj_execute_noalloc_c2c(int dtype, int64_t n, int64_t batch, int dir, double scale,
                                        const void* d_in, void* d_out, void* stream) {
  using namespace fftj;
  if (dtype != FFTJ_F32 && dtype != FFTJ_F64) {
    set_error("fftj_execute_noalloc_c2c: dtype must be F32 or F64");
    return FFTJ_ERR_ARG;
  }
  if (n < 1 || batch < 1 || (dir != -1 && dir != 1) || !d_in || !d_out) {
    set_error("fftj_execute_noalloc_c2c: bad length, batch, direction or pointer");
    return FFTJ_ERR_ARG;
  }
  // an error left pending by earlier work on this thread is reported as such
  // (and left pending) rather than blamed on this call's launches
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess) {
    set_error("fftj_execute_noalloc_c2c: a CUDA error from earlier work is pending on this thread");
    return FFTJ_ERR_CUDA;
  }
  cudaStream_t st = (cudaStream_t)stream;
  return dtype == FFTJ_F32 ? run_noalloc<float>(n, batch, dir, scale, d_in, d_out, st)
                           : run_noalloc<double>(n, batch, dir, scale, d_in, d_out, st);
}
