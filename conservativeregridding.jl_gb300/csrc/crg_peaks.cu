// crg_peaks.cu -- the FP64 arithmetic peak of the current GPU, measured with
// our own kernel: the denominator of the build's roofline (the per-pair clip
// and area is FP64 work).  Built as its own small library (libcrg_peaks.so),
// not part of the regridding ABI.
//
// k_fp64_fma: every thread runs kChains independent FMA chains
// x <- fma(x, a, b) for `iters` steps (2 FLOPs each), on a grid of
// blocks_per_sm x 256 threads per SM, so the FP64 pipe of every SM stays busy
// whatever its issue latency.  The chains stay bounded (|a| < 1) and their sum
// is stored (to one device variable) only under a condition the host makes
// false -- the chains stay non-negative and `never` is -1 -- so nothing is
// optimised away and the kernel writes nothing.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int kChains = 8;

__device__ double g_sink;

__global__ void __launch_bounds__(256) k_fp64_fma(int iters, double a, double b, double never) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = (double)(threadIdx.x + c) * 1e-6;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == never) g_sink = s;
}

}  // namespace

extern "C" {

// Best of `reps` timed launches (after one warm-up launch) of the FMA loop on
// the current device, in FP64 TFLOP/s.  Returns 0 on success, else the CUDA
// error code.
int crg_peak_fp64_tflops(int reps, double* tflops, double* ms_best) {
  if (reps < 1) reps = 1;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return (int)e;
  const int threads = 256, blocks = sms * 8, iters = 2048;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0.f;
  for (int r = 0; r <= reps; ++r) {
    cudaEventRecord(e0);
    k_fp64_fma<<<blocks, threads>>>(iters, 0.999999, 1e-7, -1.0);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && (best == 0.f || ms < best)) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return (int)e;
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  const double flops = 2.0 * kChains * (double)iters * (double)threads * (double)blocks;
  *tflops = flops / (best * 1e-3) / 1e12;
  if (ms_best) *ms_best = best;
  return 0;
}

}  // extern "C"
