// gpr.cu - sparse GPR energy and dE/dG on the CUDA cores (FP64 and FP32).
//
// Reference: GET_COV and the energy / dE/dG loops of FGAP_CALC,
// gappy/libgap/gap_calc.f90:143-166, 268-288:
//   K_ik   = exp(-0.5 * sum_d ((x_id - m_kd) / theta_d)^2)      (delta = 1)
//   e_i    = sum_k K_ik c_k,   E = sum_i e_i
//   dedg_id = -sum_k (x_id - m_kd) / theta_d^2 * K_ik c_k
// With x' = x / theta and m' = m / theta (m' precomputed at model load):
//   K_ik = exp(-0.5 |x'_i - m'_k|^2),  dedg_id = -(1/theta_d) sum_k (x'_id - m'_kd) w_ik,
// w_ik = K_ik c_k.  The differences are formed directly (no |x|^2+|m|^2-2x.m
// expansion), so there is no cancellation beyond the reference's own.
//
// Block = 32 atoms x a range of sparse points; tiles of 64 sparse points are
// staged in shared memory.  Phase A: each thread forms 8 (atom, point) kernel
// values; phase B: each thread accumulates 8 descriptor components of dE/dG.
// Small batches split the sparse points over blockIdx.y and a fixed-order
// reduction sums the partial results (deterministic).
#include <type_traits>

#include "gapgb_internal.h"

namespace gapgb {
namespace {

constexpr int kBM = 32;
constexpr int kBK = 64;
constexpr int kMaxV = 16;  // D <= 8 * kMaxV

__device__ __forceinline__ double g_exp(double x) { return exp(x); }
__device__ __forceinline__ float g_exp(float x) { return expf(x); }

template <typename T>
__global__ void __launch_bounds__(256)
    k_gpr(int N, int M, int D, int klen, const T *__restrict__ G, const T *__restrict__ mmt,
          const T *__restrict__ invth, const T *__restrict__ coeff, double *__restrict__ e_out,
          T *__restrict__ dedg_out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T *xs = reinterpret_cast<T *>(smraw);     // [kBM][D+1]
  T *ms = xs + kBM * (D + 1);               // [kBK][D+1]
  T *ws = ms + kBK * (D + 1);               // [kBM][kBK+1]
  const int t = threadIdx.x;
  const int i0 = blockIdx.x * kBM;
  const int kbeg = blockIdx.y * klen;
  const int kend = min(M, kbeg + klen);
  for (int q = t; q < kBM * D; q += 256) {
    const int r = q / D, d = q - r * D;
    const int i = i0 + r;
    xs[r * (D + 1) + d] = (i < N) ? G[(size_t)i * D + d] * invth[d] : (T)0;
  }
  const int ia = t >> 3, sub = t & 7;
  double epart = 0.0;
  T acc[kMaxV];
  T xr[kMaxV];
#pragma unroll
  for (int v = 0; v < kMaxV; ++v) acc[v] = (T)0;
  __syncthreads();
#pragma unroll
  for (int v = 0; v < kMaxV; ++v) {
    const int d = sub + 8 * v;
    xr[v] = (d < D) ? xs[ia * (D + 1) + d] : (T)0;
  }
  for (int k0 = kbeg; k0 < kend; k0 += kBK) {
    for (int q = t; q < kBK * D; q += 256) {
      const int r = q / D, d = q - r * D;
      const int k = k0 + r;
      ms[r * (D + 1) + d] = (k < kend) ? mmt[(size_t)k * D + d] : (T)0;
    }
    __syncthreads();
    // phase A: kernel values
    const T *xrow = xs + ia * (D + 1);
#pragma unroll 2
    for (int u = 0; u < kBK / 8; ++u) {
      const int kk = sub + 8 * u;
      const T *mrow = ms + kk * (D + 1);
      T s = (T)0;
#pragma unroll 4
      for (int d = 0; d < D; ++d) {
        const T df = xrow[d] - mrow[d];
        s += df * df;
      }
      const int k = k0 + kk;
      T w = (T)0;
      if (k < kend) w = g_exp((T)-0.5 * s) * coeff[k];
      ws[ia * (kBK + 1) + kk] = w;
      epart += (double)w;
    }
    __syncthreads();
    // phase B: dE/dG partial sums
    const T *wrow = ws + ia * (kBK + 1);
    const int kn = min(kBK, kend - k0);
    for (int kk = 0; kk < kn; ++kk) {
      const T w = wrow[kk];
      const T *mrow = ms + kk * (D + 1);
#pragma unroll
      for (int v = 0; v < kMaxV; ++v) {
        const int d = sub + 8 * v;
        if (d < D) acc[v] += (xr[v] - mrow[d]) * w;
      }
    }
    __syncthreads();
  }
  epart += __shfl_xor_sync(0xffffffffu, epart, 1);
  epart += __shfl_xor_sync(0xffffffffu, epart, 2);
  epart += __shfl_xor_sync(0xffffffffu, epart, 4);
  const int i = i0 + ia;
  if (i < N) {
    const size_t base = (size_t)blockIdx.y * N + i;
    if (sub == 0) e_out[base] = epart;
#pragma unroll
    for (int v = 0; v < kMaxV; ++v) {
      const int d = sub + 8 * v;
      if (d < D) dedg_out[base * D + d] = -acc[v] * invth[d];
    }
  }
}

template <typename T>
__global__ void k_gpr_reduce(int N, int D, int nsplit, const double *__restrict__ e_part,
                             const T *__restrict__ dedg_part, double *__restrict__ e,
                             T *__restrict__ dedg) {
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nd = (size_t)N * D;
  if (tid < nd) {
    T s = (T)0;
    for (int p = 0; p < nsplit; ++p) s += dedg_part[(size_t)p * nd + tid];
    dedg[tid] = s;
  }
  if (tid < (size_t)N) {
    double s = 0.0;
    for (int p = 0; p < nsplit; ++p) s += e_part[(size_t)p * N + tid];
    e[tid] = s;
  }
}

}  // namespace

int gpr_nsplit(int N, int M) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int bx = (N + kBM - 1) / kBM;
  const int kt = (M + kBK - 1) / kBK;
  int ns = (2 * sms + bx - 1) / bx;
  if (ns < 1) ns = 1;
  if (ns > kt) ns = kt;
  return ns;
}

size_t gpr_scratch_bytes(int N, int M, int D, size_t elem) {
  const int ns = gpr_nsplit(N, M);
  if (ns <= 1) return 0;
  return (size_t)ns * N * sizeof(double) + (size_t)ns * N * D * elem;
}

template <typename T>
void launch_gpr(const gapgb_model *m, Workspace &ws, int N, cudaStream_t st) {
  const int M = m->host.M, D = m->host.D;
  const int ns = gpr_nsplit(N, M);
  const int kt = (M + kBK - 1) / kBK;
  const int klen = ((kt + ns - 1) / ns) * kBK;
  const int nsp = (M + klen - 1) / klen;
  const size_t smem = ((size_t)(kBM + kBK) * (D + 1) + (size_t)kBM * (kBK + 1)) * sizeof(T);
  auto fn = k_gpr<T>;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const T *mmt = std::is_same<T, double>::value ? (const T *)m->d_mmt : (const T *)m->d_mmt32;
  const T *invth = std::is_same<T, double>::value ? (const T *)m->d_invth : (const T *)m->d_invth32;
  const T *coeff = std::is_same<T, double>::value ? (const T *)m->d_coeff : (const T *)m->d_coeff32;
  dim3 grid((N + kBM - 1) / kBM, nsp);
  if (nsp == 1) {
    fn<<<grid, 256, smem, st>>>(N, M, D, klen, (const T *)ws.G, mmt, invth, coeff, ws.e,
                                (T *)ws.dedg);
  } else {
    double *e_part = reinterpret_cast<double *>(ws.gpr_scratch);
    T *d_part = reinterpret_cast<T *>(e_part + (size_t)nsp * N);
    fn<<<grid, 256, smem, st>>>(N, M, D, klen, (const T *)ws.G, mmt, invth, coeff, e_part, d_part);
    const size_t nd = (size_t)N * D;
    k_gpr_reduce<T><<<(unsigned)((nd + 255) / 256), 256, 0, st>>>(N, D, nsp, e_part, d_part, ws.e,
                                                                    (T *)ws.dedg);
  }
}

template void launch_gpr<double>(const gapgb_model *, Workspace &, int, cudaStream_t);
template void launch_gpr<float>(const gapgb_model *, Workspace &, int, cudaStream_t);

}  // namespace gapgb
