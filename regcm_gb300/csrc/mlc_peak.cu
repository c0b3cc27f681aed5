// mlc_peak.cu -- FP64 throughput of this GPU, measured the way the FP64 step
// uses the FP64 pipe (the plain FP64 path's bound on GB300, where FP64 runs
// at a small fraction of the FP32 rate).
//
// Every thread runs C independent multiply-add chains a = a*x + y (x just
// below one, so nothing grows or underflows), long enough that launch
// overhead is negligible.  A few chain counts and blocks per SM are tried
// (latency hiding by chains within a thread or by resident warps); each is
// timed with CUDA events on a private stream, best of `repeats` launches
// after one warm-up, and the fastest rate is returned, in FLOP/s counting a
// multiply-add as two.
#include <cuda_runtime.h>

#include "../../include/moloch_gb300.h"

namespace {

constexpr int kThreads = 256;

// the chains' sum lands here only if it equals -1, which it never does (the
// chains converge to y / (1 - x) = 1); the store keeps them from being removed
__device__ double g_fma_sink;

template <int C>
__global__ void __launch_bounds__(kThreads) k_fp64_fma(int iters, double x, double y) {
  double a[C];
#pragma unroll
  for (int c = 0; c < C; ++c) a[c] = 1.0 + 1e-3 * (threadIdx.x + c);
#pragma unroll 4
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < C; ++c) a[c] = __fma_rn(a[c], x, y);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < C; ++c) s += a[c];
  if (s == -1.0) g_fma_sink = s;
}

template <int C>
int time_config(cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, int blocks, int iters, int repeats,
                double *rate) {
  float best = 0.0f;
  for (int r = 0; r <= repeats; ++r) {
    cudaEventRecord(e0, s);
    k_fp64_fma<C><<<blocks, kThreads, 0, s>>>(iters, 0.9999999, 1e-7);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) return MLC_ERR_CUDA;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && (best == 0.0f || ms < best)) best = ms;
  }
  if (cudaGetLastError() != cudaSuccess) return MLC_ERR_CUDA;
  const double fmas = (double)blocks * kThreads * (double)iters * C;
  *rate = 2.0 * fmas / (best * 1e-3);
  return MLC_OK;
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
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    if (s) cudaStreamDestroy(s);
    if (e0) cudaEventDestroy(e0);
    return MLC_ERR_CUDA;
  }
  double best = 0.0;
  int st = MLC_OK;
  // 2, 4 and 8 blocks of 256 threads an SM (8: one full wave of 2048
  // threads), each with 4, 8 or 16 chains a thread; the same multiply-adds a
  // thread for every chain count
  const int per_sm[3] = {2, 4, 8};
  for (int q = 0; q < 3 && st == MLC_OK; ++q) {
    double r4 = 0.0, r8 = 0.0, r16 = 0.0;
    st = time_config<4>(s, e0, e1, sms * per_sm[q], 16384, repeats, &r4);
    if (st == MLC_OK) st = time_config<8>(s, e0, e1, sms * per_sm[q], 8192, repeats, &r8);
    if (st == MLC_OK) st = time_config<16>(s, e0, e1, sms * per_sm[q], 4096, repeats, &r16);
    best = best > r4 ? best : r4;
    best = best > r8 ? best : r8;
    best = best > r16 ? best : r16;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  if (st != MLC_OK) return st;
  *flops = best;
  return MLC_OK;
}
