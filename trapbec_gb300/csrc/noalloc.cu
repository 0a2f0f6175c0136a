// noalloc.cu -- the norm / |psi| statistics reduction with no allocation.
//
// trapbec_psi_stats_noalloc computes what trapbec_diag reports as intpsi2,
// maxpsi, minpsi and meanpsi (the reference's Psi_norm and Psi_info) for a
// psi array the caller already holds on the device, and writes the four
// values to device memory the caller provides.  It calls no cudaMalloc,
// cudaFree or other allocating routine.  Its scratch space -- one set of
// per-block partial sums -- is the file-scope device array below, which every
// GPU that loads the library holds until the process exits.
//
// It exists for callers that cannot let a library allocate device memory:
// hosts that reserve all of a GPU's memory up front in their own pool (a
// framework's caching allocator, or a Fortran code that sizes everything at
// start-up) and must not have a library take memory behind the pool's back
// or stall their other streams with the device synchronisation cudaMalloc
// and cudaFree may perform.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/trapbec.h"
#include "host_util.h"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_CELLS_PER_THREAD = 64;
constexpr long long NA_CELLS_PER_BLOCK = (long long)NA_THREADS * NA_CELLS_PER_THREAD;  // 16384
constexpr int NA_MAX_BLOCKS = 16384;
constexpr int NA_NQ = 4;  // sum|psi|^2, max|psi|, min|psi|, sum|psi|

// The scratch: NA_MAX_BLOCKS x 4 doubles = 512 KiB, 256-byte aligned.  Every
// call overwrites the slots of the blocks it launches before reading them, so
// nothing has to start at zero; the contents left by the previous call are
// never read.
static __device__ __align__(256) double g_noalloc_scratch[NA_MAX_BLOCKS * NA_NQ];

// Per-device address of g_noalloc_scratch and the unique id of the CUDA
// context it was looked up in.  The array is part of the library's module,
// which is loaded into each context separately: after the caller resets the
// device (cudaDeviceReset) or releases and re-creates its primary context,
// the module is loaded again and the array can sit at another address, so
// the address is looked up again whenever the current context's id changes.
constexpr int NA_MAX_DEVICES = 64;
void* g_scratch_addr[NA_MAX_DEVICES] = {nullptr};
unsigned long long g_scratch_ctx[NA_MAX_DEVICES] = {0};
std::mutex g_scratch_mu;

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points
// (the library links the static runtime, not libcuda).
using PFN_ctx_get_current = CUresult (*)(CUcontext*);
using PFN_ctx_get_id = CUresult (*)(CUcontext, unsigned long long*);

template <typename F> F driver_fn(const char* name) {
  void* f = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return reinterpret_cast<F>(f);
}

// Unique id of the calling thread's current context (0 if it cannot be read).
unsigned long long current_ctx_id() {
  static PFN_ctx_get_current get_cur = driver_fn<PFN_ctx_get_current>("cuCtxGetCurrent");
  static PFN_ctx_get_id get_id = driver_fn<PFN_ctx_get_id>("cuCtxGetId");
  if (!get_cur || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_cur(&ctx) != CUDA_SUCCESS || ctx == nullptr) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

template <typename T> struct C2;
template <> struct C2<float> { using t = float2; };
template <> struct C2<double> { using t = double2; };

// Pass 1: block b reduces cells [b * NA_CELLS_PER_BLOCK, (b+1) * NA_CELLS_PER_BLOCK)
// and writes its four partials to scratch[4 b .. 4 b + 3].
template <typename T>
__global__ void __launch_bounds__(NA_THREADS) stats_partial_kernel(const typename C2<T>::t* __restrict__ psi,
                                                                    long long n, double* __restrict__ scratch) {
  const long long base = (long long)blockIdx.x * NA_CELLS_PER_BLOCK;
  double s2 = 0.0, s1 = 0.0;
  double mx = 0.0, mn = 1.0e300;
  for (int k = 0; k < NA_CELLS_PER_THREAD; ++k) {
    const long long i = base + (long long)k * NA_THREADS + threadIdx.x;
    if (i < n) {
      const typename C2<T>::t v = psi[i];
      const double re = (double)v.x, im = (double)v.y;
      const double a2 = re * re + im * im;
      const double a = sqrt(a2);
      s2 += a2;
      s1 += a;
      mx = fmax(mx, a);
      mn = fmin(mn, a);
    }
  }
  __shared__ double sh[NA_NQ][NA_THREADS];
  sh[0][threadIdx.x] = s2;
  sh[1][threadIdx.x] = mx;
  sh[2][threadIdx.x] = mn;
  sh[3][threadIdx.x] = s1;
  __syncthreads();
  for (int w = NA_THREADS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      const int j = threadIdx.x + w;
      sh[0][threadIdx.x] += sh[0][j];
      sh[1][threadIdx.x] = fmax(sh[1][threadIdx.x], sh[1][j]);
      sh[2][threadIdx.x] = fmin(sh[2][threadIdx.x], sh[2][j]);
      sh[3][threadIdx.x] += sh[3][j];
    }
    __syncthreads();
  }
  if (threadIdx.x < NA_NQ) scratch[(size_t)blockIdx.x * NA_NQ + threadIdx.x] = sh[threadIdx.x][0];
}

// Pass 2 (one block): combine the nblk partials in a fixed order and write
// out[0..3] = intpsi2, maxpsi, minpsi, meanpsi.
__global__ void __launch_bounds__(NA_THREADS) stats_final_kernel(const double* __restrict__ scratch, int nblk,
                                                                 long long n, double* __restrict__ out) {
  double s2 = 0.0, s1 = 0.0, mx = 0.0, mn = 1.0e300;
  for (int b = threadIdx.x; b < nblk; b += NA_THREADS) {
    s2 += scratch[(size_t)b * NA_NQ + 0];
    mx = fmax(mx, scratch[(size_t)b * NA_NQ + 1]);
    mn = fmin(mn, scratch[(size_t)b * NA_NQ + 2]);
    s1 += scratch[(size_t)b * NA_NQ + 3];
  }
  __shared__ double sh[NA_NQ][NA_THREADS];
  sh[0][threadIdx.x] = s2;
  sh[1][threadIdx.x] = mx;
  sh[2][threadIdx.x] = mn;
  sh[3][threadIdx.x] = s1;
  __syncthreads();
  for (int w = NA_THREADS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      const int j = threadIdx.x + w;
      sh[0][threadIdx.x] += sh[0][j];
      sh[1][threadIdx.x] = fmax(sh[1][threadIdx.x], sh[1][j]);
      sh[2][threadIdx.x] = fmin(sh[2][threadIdx.x], sh[2][j]);
      sh[3][threadIdx.x] += sh[3][j];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sh[0][0];
    out[1] = sh[1][0];
    out[2] = sh[2][0];
    out[3] = sh[3][0] / (double)n;
  }
}

// Device address of the scratch array for the current device; looked up the
// first time this device is used (with the device current) and again when the
// device's context has changed since, remembered otherwise.
int scratch_for_current_device(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    tbh::set_error(std::string("trapbec_psi_stats_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return TRAPBEC_ERR_NODEVICE;
  }
  if (dev < 0 || dev >= NA_MAX_DEVICES) {
    tbh::set_error("trapbec_psi_stats_noalloc: device ordinal out of range");
    return TRAPBEC_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  unsigned long long ctx = current_ctx_id();
  if (g_scratch_addr[dev] == nullptr || ctx == 0 || ctx != g_scratch_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      tbh::set_error(std::string("trapbec_psi_stats_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return TRAPBEC_ERR_CUDA;
    }
    // the lookup made the device's primary context current if none was
    if (ctx == 0) ctx = current_ctx_id();
    g_scratch_addr[dev] = p;
    g_scratch_ctx[dev] = ctx;
  }
  *out = static_cast<double*>(g_scratch_addr[dev]);
  return TRAPBEC_OK;
}

}  // namespace

extern "C" int trapbec_psi_stats_noalloc(const void* psi, int64_t ncells, int precision, double* stats,
                                         void* stream) {
  if (!psi || !stats) {
    tbh::set_error("trapbec_psi_stats_noalloc: null pointer");
    return TRAPBEC_ERR_ARG;
  }
  if (precision != TRAPBEC_FP32 && precision != TRAPBEC_FP64) {
    tbh::set_error("trapbec_psi_stats_noalloc: precision must be TRAPBEC_FP32 or TRAPBEC_FP64");
    return TRAPBEC_ERR_ARG;
  }
  // the kernels read psi as float2 / double2 and write stats as doubles: a
  // pointer off that alignment would fault on the device, so refuse it here
  const uintptr_t palign = precision == TRAPBEC_FP64 ? 16u : 8u;
  if (reinterpret_cast<uintptr_t>(psi) % palign != 0) {
    tbh::set_error("trapbec_psi_stats_noalloc: psi must be aligned to " + std::to_string((unsigned)palign) +
                   " bytes (one complex value of the precision)");
    return TRAPBEC_ERR_ARG;
  }
  if (reinterpret_cast<uintptr_t>(stats) % 8u != 0) {
    tbh::set_error("trapbec_psi_stats_noalloc: stats must be aligned to 8 bytes (double)");
    return TRAPBEC_ERR_ARG;
  }
  const long long max_cells = NA_CELLS_PER_BLOCK * (long long)NA_MAX_BLOCKS;
  if (ncells <= 0 || ncells > max_cells) {
    tbh::set_error("trapbec_psi_stats_noalloc: ncells must be in 1.." + std::to_string(max_cells) +
                   " (the fixed scratch holds " + std::to_string(NA_MAX_BLOCKS) + " block partials of " +
                   std::to_string(NA_CELLS_PER_BLOCK) + " cells each); got " + std::to_string((long long)ncells));
    return TRAPBEC_ERR_ARG;
  }
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nblk = (int)((ncells + NA_CELLS_PER_BLOCK - 1) / NA_CELLS_PER_BLOCK);
  if (precision == TRAPBEC_FP64)
    stats_partial_kernel<double><<<nblk, NA_THREADS, 0, st>>>(static_cast<const double2*>(psi), ncells, scratch);
  else
    stats_partial_kernel<float><<<nblk, NA_THREADS, 0, st>>>(static_cast<const float2*>(psi), ncells, scratch);
  stats_final_kernel<<<1, NA_THREADS, 0, st>>>(scratch, nblk, ncells, stats);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    tbh::set_error(std::string("trapbec_psi_stats_noalloc: launch: ") + cudaGetErrorString(e));
    return TRAPBEC_ERR_CUDA;
  }
  return TRAPBEC_OK;
}
