// peaks.cu -- measured FP64 instruction rate of the GPU, the compute roofline
// of the FP64 stage kernels (no counterpart in the reference).
//
// GB300 issues FP64 at a small fraction of its FP32 rate, so the FP64 stage
// kernels are bound by the FP64 pipe rather than by HBM.  Their roofline is
// the rate at which the SMs retire DFMA instructions: every thread of a grid
// of 8 CTAs per SM runs 8 independent FMA chains (enough instructions in
// flight to cover the pipe's latency), and the launch is timed with CUDA
// events after one warm-up launch.
#include <cuda_runtime.h>

#include <string>

#include "../../include/trapbec.h"
#include "host_util.h"

namespace {

constexpr int PK_THREADS = 256;
constexpr int PK_CHAINS = 8;

__global__ void __launch_bounds__(PK_THREADS) fp64_fma_chains_kernel(double* out, int iters, double b, double c) {
  double a[PK_CHAINS];
#pragma unroll
  for (int k = 0; k < PK_CHAINS; ++k) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < PK_CHAINS; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < PK_CHAINS; ++k) s += a[k];
  if (s == -1.0) out[blockIdx.x] = s;   // never true: keeps the chains from being removed
}

}  // namespace

extern "C" int trapbec_fp64_fma_rate(double* ops_per_second) {
  if (!ops_per_second) return TRAPBEC_ERR_ARG;
  int dev = 0, nsm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) {
    tbh::set_error(std::string("trapbec_fp64_fma_rate: ") + cudaGetErrorString(e));
    return TRAPBEC_ERR_NODEVICE;
  }
  const int grid = nsm * 8;
  const int iters = 1 << 14;
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float ms = 0.f;
  e = cudaMalloc(&out, sizeof(double) * grid);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    fp64_fma_chains_kernel<<<grid, PK_THREADS>>>(out, iters, 0.999999, 1e-7);   // warm-up
    cudaEventRecord(e0);
    fp64_fma_chains_kernel<<<grid, PK_THREADS>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  if (e != cudaSuccess || !(ms > 0.f)) {
    tbh::set_error(std::string("trapbec_fp64_fma_rate: ") + cudaGetErrorString(e));
    return TRAPBEC_ERR_CUDA;
  }
  *ops_per_second = (double)grid * PK_THREADS * PK_CHAINS * (double)iters / (ms * 1e-3);
  return TRAPBEC_OK;
}
