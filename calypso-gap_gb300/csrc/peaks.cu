// peaks.cu - measured arithmetic peaks of the current GPU.
//
// The roofline denominators of the descriptor, chain-rule and plain-FP64
// kernels: the FP32 FMA rate, the FP64 FMA rate and the MUFU ex2 rate of the
// device, each measured by a kernel that keeps every SM busy with
// independent dependency chains of that one operation (8 blocks of 256
// threads per SM, 8 chains per thread), timed with CUDA events after a
// warm-up launch.  Block 0 also reads the SM cycle counter around its work,
// which gives the clock the kernel ran at (cycles / event time).
#include "gapgb_internal.h"

namespace gapgb {
namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kThreads) k_peak_fma(int iters, T b, T c, T *sink,
                                                       long long *cycles) {
  T a[kChains];
#pragma unroll
  for (int q = 0; q < kChains; ++q) a[q] = (T)(threadIdx.x + q);
  const long long t0 = clock64();
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int q = 0; q < kChains; ++q) a[q] = fma(a[q], b, c);
  }
  const long long t1 = clock64();
  T s = 0;
#pragma unroll
  for (int q = 0; q < kChains; ++q) s += a[q];
  if (s == (T)-12345.678) sink[0] = s;  // never true for the chosen b, c: keeps the chains live
  if (blockIdx.x == 0 && threadIdx.x == 0) cycles[0] = t1 - t0;
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// x <- 2^(-x) converges to the fixed point 0.6412, so the chains stay finite
__global__ void __launch_bounds__(kThreads) k_peak_ex2(int iters, float *sink, long long *cycles) {
  float a[kChains];
#pragma unroll
  for (int q = 0; q < kChains; ++q) a[q] = 0.01f * (float)(threadIdx.x & 7) + 0.1f * q;
  const long long t0 = clock64();
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int q = 0; q < kChains; ++q) a[q] = ex2_approx(-a[q]);
  }
  const long long t1 = clock64();
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < kChains; ++q) s += a[q];
  if (s < 0.f) sink[0] = s;
  if (blockIdx.x == 0 && threadIdx.x == 0) cycles[0] = t1 - t0;
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

extern "C" gapgb_status gapgb_measure_peaks(double out[6]) {
  if (!out) return GAPGB_ERR_ARG;
  int dev = 0, sms = 0;
  GAPGB_CUDA_TRY(cudaGetDevice(&dev));
  GAPGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8;
  const double threads = (double)blocks * kThreads;
  void *buf = nullptr;
  GAPGB_CUDA_TRY(cudaMalloc(&buf, 256));
  double *sink = static_cast<double *>(buf);
  long long *cyc = reinterpret_cast<long long *>(static_cast<char *>(buf) + 128);
  long long h_cyc = 0;
  float ms = 0.f;
  gapgb_status st = GAPGB_OK;
  // FP32 FMA: an FMA counts two flops
  const int it32 = 16384;
  st = time_kernel([&] {
    k_peak_fma<float><<<blocks, kThreads>>>(it32, 0.999999f, 1e-7f, (float *)sink, cyc);
  }, &ms);
  if (st == GAPGB_OK) {
    out[0] = threads * it32 * 8 * kChains * 2.0 / (ms * 1e-3) / 1e12;
    cudaMemcpy(&h_cyc, cyc, sizeof(h_cyc), cudaMemcpyDeviceToHost);
    out[3] = (double)h_cyc / (ms * 1e-3) / 1e6;
  }
  // FP64 FMA
  const int it64 = 512;
  if (st == GAPGB_OK)
    st = time_kernel([&] {
      k_peak_fma<double><<<blocks, kThreads>>>(it64, 0.999999999, 1e-12, sink, cyc);
    }, &ms);
  if (st == GAPGB_OK) {
    out[1] = threads * it64 * 8 * kChains * 2.0 / (ms * 1e-3) / 1e12;
    cudaMemcpy(&h_cyc, cyc, sizeof(h_cyc), cudaMemcpyDeviceToHost);
    out[4] = (double)h_cyc / (ms * 1e-3) / 1e6;
  }
  // MUFU ex2, in units of 1e12 per second
  const int itx = 2048;
  if (st == GAPGB_OK)
    st = time_kernel([&] { k_peak_ex2<<<blocks, kThreads>>>(itx, (float *)sink, cyc); }, &ms);
  if (st == GAPGB_OK) {
    out[2] = threads * itx * 8 * kChains / (ms * 1e-3) / 1e12;
    cudaMemcpy(&h_cyc, cyc, sizeof(h_cyc), cudaMemcpyDeviceToHost);
    out[5] = (double)h_cyc / (ms * 1e-3) / 1e6;
  }
  cudaFree(buf);
  return st;
}
