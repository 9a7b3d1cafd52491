// peaks.cu - measured arithmetic peaks of the current GPU.
//
// The roofline denominators of the descriptor, chain-rule and plain-FP64
// kernels: the FP32 FMA rate, the FP64 FMA rate and the MUFU ex2 rate of the
// device, each measured by a kernel that keeps every SM busy with
// independent dependency chains of that one operation (one resident wave of
// 256-thread blocks, as many per SM as fit, 8 chains per thread), timed with
// CUDA events after a warm-up launch.  The clock the rates were taken at is
// the caller's to sample (nvidia-smi), as for every other timed region.
#include "gapgb_internal.h"

namespace gapgb {
namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kThreads) k_peak_fma(int iters, T b, T c, T *sink) {
  T a[kChains];
#pragma unroll
  for (int q = 0; q < kChains; ++q) a[q] = (T)(threadIdx.x + q);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int q = 0; q < kChains; ++q) a[q] = fma(a[q], b, c);
  }
  T s = 0;
#pragma unroll
  for (int q = 0; q < kChains; ++q) s += a[q];
  if (s == (T)-12345.678) sink[0] = s;  // never true for the chosen b, c: keeps the chains live
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// x <- 2^(-x) converges to the fixed point 0.6412, so the chains stay finite
__global__ void __launch_bounds__(kThreads) k_peak_ex2(int iters, float *sink) {
  float a[kChains];
#pragma unroll
  for (int q = 0; q < kChains; ++q) a[q] = 0.01f * (float)(threadIdx.x & 7) + 0.1f * q;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int q = 0; q < kChains; ++q) a[q] = ex2_approx(-a[q]);
  }
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < kChains; ++q) s += a[q];
  if (s < 0.f) sink[0] = s;
}

template <typename Launch>
gapgb_status time_kernel(Launch launch, float *ms) {
  cudaEvent_t a, b;
  GAPGB_CUDA_TRY(cudaEventCreate(&a));
  GAPGB_CUDA_TRY(cudaEventCreate(&b));
  launch();  // warm-up
  GAPGB_CUDA_TRY(cudaGetLastError());
  GAPGB_CUDA_TRY(cudaEventRecord(a, 0));
  launch();
  GAPGB_CUDA_TRY(cudaEventRecord(b, 0));
  GAPGB_CUDA_TRY(cudaEventSynchronize(b));
  GAPGB_CUDA_TRY(cudaGetLastError());
  GAPGB_CUDA_TRY(cudaEventElapsedTime(ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return GAPGB_OK;
}

}  // namespace
}  // namespace gapgb

using namespace gapgb;

extern "C" gapgb_status gapgb_measure_peaks(double out[3]) {
  if (!out) return GAPGB_ERR_ARG;
  int dev = 0, sms = 0;
  GAPGB_CUDA_TRY(cudaGetDevice(&dev));
  GAPGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // one resident wave per kernel: blocks = SMs x the blocks that fit on one
  int occ[3] = {1, 1, 1};
  GAPGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[0], k_peak_fma<float>,
                                                               kThreads, 0));
  GAPGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[1], k_peak_fma<double>,
                                                               kThreads, 0));
  GAPGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[2], k_peak_ex2, kThreads, 0));
  void *buf = nullptr;
  GAPGB_CUDA_TRY(cudaMalloc(&buf, 256));
  double *sink = static_cast<double *>(buf);
  float ms = 0.f;
  gapgb_status st = GAPGB_OK;
  // FP32 FMA: an FMA counts two flops
  const int it32 = 65536, b32 = sms * (occ[0] > 0 ? occ[0] : 1);
  st = time_kernel([&] {
    k_peak_fma<float><<<b32, kThreads>>>(it32, 0.999999f, 1e-7f, (float *)sink);
  }, &ms);
  if (st == GAPGB_OK) {
    out[0] = (double)b32 * kThreads * it32 * 8 * kChains * 2.0 / (ms * 1e-3) / 1e12;
  }
  // FP64 FMA
  const int it64 = 2048, b64 = sms * (occ[1] > 0 ? occ[1] : 1);
  if (st == GAPGB_OK)
    st = time_kernel([&] {
      k_peak_fma<double><<<b64, kThreads>>>(it64, 0.999999999, 1e-12, sink);
    }, &ms);
  if (st == GAPGB_OK) {
    out[1] = (double)b64 * kThreads * it64 * 8 * kChains * 2.0 / (ms * 1e-3) / 1e12;
  }
  // MUFU ex2, in units of 1e12 per second
  const int itx = 8192, bx = sms * (occ[2] > 0 ? occ[2] : 1);
  if (st == GAPGB_OK)
    st = time_kernel([&] { k_peak_ex2<<<bx, kThreads>>>(itx, (float *)sink); }, &ms);
  if (st == GAPGB_OK) {
    out[2] = (double)bx * kThreads * itx * 8 * kChains / (ms * 1e-3) / 1e12;
  }
  cudaFree(buf);
  return st;
}
