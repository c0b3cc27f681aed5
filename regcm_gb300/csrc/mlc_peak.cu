// mlc_peak.cu -- FP64 throughput of this GPU, measured the way the FP64 step
// uses the FP64 pipe (the plain FP64 path's bound on GB300, where FP64 runs
// at a small fraction of the FP32 rate).
//
// Every thread runs kChains independent multiply-add chains
// a = a*x + y (x just below one, so nothing grows or underflows), long
// enough that launch overhead is negligible; blocks fill every SM several
// times over.  The result is the best of `repeats` launches, timed with CUDA
// events on a private stream, in FLOP/s counting a multiply-add as two.
#include <cuda_runtime.h>

#include "../../include/moloch_gb300.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

// the chains' sum lands here only if it equals -1, which it never does (the
// chains converge to y / (1 - x) = 1); the store keeps them from being removed
__device__ double g_fma_sink;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(int iters, double x, double y) {
  double a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) a[c] = 1.0 + 1e-3 * (threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = __fma_rn(a[c], x, y);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c];
  if (s == -1.0) g_fma_sink = s;
}

}  // namespace

extern "C" int mlc_fp64_peak(int repeats, double *flops) {
  if (!flops || repeats < 1) return MLC_ERR_INVALID;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return MLC_ERR_NODEVICE;
  }
  const int blocks = sms * 16;
  const int iters = 4096;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    if (s) cudaStreamDestroy(s);
    if (e0) cudaEventDestroy(e0);
    return MLC_ERR_CUDA;
  }
  float best = 0.0f;
  int st = MLC_OK;
  // one warm-up launch, then the timed ones
  for (int r = 0; r <= repeats && st == MLC_OK; ++r) {
    cudaEventRecord(e0, s);
    k_fp64_fma<<<blocks, kThreads, 0, s>>>(iters, 0.9999999, 1e-7);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      st = MLC_ERR_CUDA;
      break;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && (best == 0.0f || ms < best)) best = ms;
  }
  if (cudaGetLastError() != cudaSuccess) st = MLC_ERR_CUDA;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  if (st != MLC_OK) return st;
  const double fmas = (double)blocks * kThreads * (double)iters * kChains;
  *flops = 2.0 * fmas / (best * 1e-3);
  return MLC_OK;
}
