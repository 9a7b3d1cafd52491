// gpr_noalloc.cu - the sparse-GPR step with no device allocation.
//
// gapgb_gpr_noalloc computes atomic energies and dE/dG (FP64) for descriptors
// that are already in device memory, using only memory that exists before
// the call: the model's resident arrays, the caller's input and output
// buffers, and one file-scope scratch array in device memory.  It is meant
// for callers that cannot call cudaMalloc at the point where they need the
// energies: host programs (simulation engines, serving processes) that
// reserve all device memory up front in their own pool, so a cudaMalloc
// behind their back fails or eats into that pool, and latency-critical loops
// that cannot afford the device-wide synchronisation cudaMalloc / cudaFree
// may cause.
//
// The scratch array holds the partial sums of the split over sparse points
// (the same split as the regular GPR kernel) and is a fixed 8 MiB
// (kNoAllocScratch doubles) per GPU that loads the library, kept until the
// process exits.  A call needs splits * natoms * (des_len + 1) doubles and is
// rejected with GAPGB_ERR_CAP_EXCEEDED when even one split does not fit,
// i.e. when natoms * (des_len + 1) > kNoAllocScratch (16131 atoms at D = 64).
// Every call shares the array and leaves its partial sums behind; each call
// writes every entry before reading it, so nothing needs clearing, but calls
// that overlap on the GPU (other streams or host threads) race on it and must
// be serialised by the caller.
//
// Set-up, once per device, is done by the first call on that device with
// that device current: the device address of the array (cudaGetSymbolAddress;
// in host code the array's name is only a host-side stand-in) and the
// kernel's shared-memory limit for the largest descriptor length.  The
// coefficients are read from the model's device copy: finish (synchronise)
// every call of this entry point before gapgb_model_set_coeff rewrites them.
#include <mutex>

#include "gapgb_internal.h"

namespace gapgb {
namespace {

constexpr size_t kNoAllocScratch = size_t(1) << 20;  // doubles (8 MiB)
constexpr int kNBM = 32;                              // atoms per block
constexpr int kNBK = 64;                              // sparse points per tile
constexpr int kNMaxV = 16;                            // D <= 8 * kNMaxV
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratch];

// shared memory of k_gpr_noalloc for descriptor length D
constexpr size_t noalloc_smem(int D) {
  return ((size_t)(kNBM + kNBK) * (D + 1) + (size_t)kNBM * (kNBK + 1)) * sizeof(double);
}

std::mutex g_ptr_mu;
double *g_ptr[kMaxDevices] = {nullptr};
int g_sms[kMaxDevices] = {0};

// FP64 GPR over a range of sparse points per blockIdx.y; partial e and
// dE/dG of split y go to part_e[y*N + i] and part_d[(y*N + i)*D + d].
__global__ void __launch_bounds__(256)
    k_gpr_noalloc(int N, int M, int D, int klen, const double *__restrict__ G,
                  const double *__restrict__ mmt, const double *__restrict__ invth,
                  const double *__restrict__ coeff, double *__restrict__ part_e,
                  double *__restrict__ part_d) {
  extern __shared__ __align__(16) unsigned char smraw[];
  double *xs = reinterpret_cast<double *>(smraw);  // [kNBM][D+1]
  double *ms = xs + kNBM * (D + 1);                 // [kNBK][D+1]
  double *ws = ms + kNBK * (D + 1);                 // [kNBM][kNBK+1]
  const int t = threadIdx.x;
  const int i0 = blockIdx.x * kNBM;
  const int kbeg = blockIdx.y * klen;
  const int kend = min(M, kbeg + klen);
  for (int q = t; q < kNBM * D; q += 256) {
    const int r = q / D, d = q - r * D;
    const int i = i0 + r;
    xs[r * (D + 1) + d] = (i < N) ? G[(size_t)i * D + d] * invth[d] : 0.0;
  }
  const int ia = t >> 3, sub = t & 7;
  double epart = 0.0, acc[kNMaxV], xr[kNMaxV];
  __syncthreads();
#pragma unroll
  for (int v = 0; v < kNMaxV; ++v) {
    const int d = sub + 8 * v;
    acc[v] = 0.0;
    xr[v] = (d < D) ? xs[ia * (D + 1) + d] : 0.0;
  }
  for (int k0 = kbeg; k0 < kend; k0 += kNBK) {
    for (int q = t; q < kNBK * D; q += 256) {
      const int r = q / D, d = q - r * D;
      const int k = k0 + r;
      ms[r * (D + 1) + d] = (k < kend) ? mmt[(size_t)k * D + d] : 0.0;
    }
    __syncthreads();
    for (int u = 0; u < kNBK / 8; ++u) {
      const int kk = sub + 8 * u;
      double s = 0.0;
      for (int d = 0; d < D; ++d) {
        const double df = xs[ia * (D + 1) + d] - ms[kk * (D + 1) + d];
        s += df * df;
      }
      const int k = k0 + kk;
      const double w = (k < kend) ? exp(-0.5 * s) * coeff[k] : 0.0;
      ws[ia * (kNBK + 1) + kk] = w;
      epart += w;
    }
    __syncthreads();
    const int kn = min(kNBK, kend - k0);
    for (int kk = 0; kk < kn; ++kk) {
      const double w = ws[ia * (kNBK + 1) + kk];
#pragma unroll
      for (int v = 0; v < kNMaxV; ++v) {
        const int d = sub + 8 * v;
        if (d < D) acc[v] += (xr[v] - ms[kk * (D + 1) + d]) * w;
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
    if (sub == 0) part_e[base] = epart;
#pragma unroll
    for (int v = 0; v < kNMaxV; ++v) {
      const int d = sub + 8 * v;
      if (d < D) part_d[base * D + d] = -acc[v] * invth[d];
    }
  }
}

// fixed-order sum of the splits into the caller's outputs
__global__ void k_gpr_noalloc_sum(int N, int D, int ns, const double *__restrict__ part_e,
                                  const double *__restrict__ part_d, double *__restrict__ e,
                                  double *__restrict__ dedg) {
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nd = (size_t)N * D;
  if (tid < nd) {
    double s = 0.0;
    for (int p = 0; p < ns; ++p) s += part_d[(size_t)p * nd + tid];
    dedg[tid] = s;
  }
  if (tid < (size_t)N) {
    double s = 0.0;
    for (int p = 0; p < ns; ++p) s += part_e[(size_t)p * N + tid];
    e[tid] = s;
  }
}

gapgb_status fail_na(gapgb_status st, const std::string &msg) {
  set_last_error(msg);
  return st;
}

}  // namespace
}  // namespace gapgb

using namespace gapgb;

extern "C" gapgb_status gapgb_gpr_noalloc(gapgb_model *m, int natoms, const double *d_G,
                                          double *d_e, double *d_dedg, void *stream) {
  if (!m || !d_G || !d_e || !d_dedg) return fail_na(GAPGB_ERR_ARG, "null argument");
  if (natoms <= 0) return fail_na(GAPGB_ERR_ARG, "natoms must be positive");
  const int M = m->host.M, D = m->host.D;
  if (D > 8 * kNMaxV) return fail_na(GAPGB_ERR_CAP_EXCEEDED, "descriptor length D > 128");
  const size_t per_split = (size_t)natoms * (size_t)(D + 1);
  if (per_split > kNoAllocScratch)
    return fail_na(GAPGB_ERR_CAP_EXCEEDED,
                   "gapgb_gpr_noalloc: natoms * (des_len + 1) = " + std::to_string(per_split) +
                       " exceeds the fixed scratch of " + std::to_string(kNoAllocScratch) +
                       " doubles");
  if (!m->d_sf)
    return fail_na(GAPGB_ERR_ARG,
                   "gapgb_gpr_noalloc: the model is not resident on the device yet (run one "
                   "evaluation first; this call does not upload it)");
  if (m->device < 0 || m->device >= kMaxDevices)
    return fail_na(GAPGB_ERR_ARG, "device ordinal out of range");
  GAPGB_CUDA_TRY(cudaSetDevice(m->device));
  double *scratch = nullptr;
  int sms = 0;
  {
    // once per device: the array's device address, the kernel's shared-memory
    // limit (for the largest D it accepts) and the SM count
    std::lock_guard<std::mutex> lock(g_ptr_mu);
    if (!g_ptr[m->device]) {
      void *p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess)
        return fail_na(GAPGB_ERR_CUDA,
                       std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      e = cudaFuncSetAttribute(k_gpr_noalloc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)noalloc_smem(8 * kNMaxV));
      if (e != cudaSuccess)
        return fail_na(GAPGB_ERR_CUDA,
                       std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
      int n = 0;
      e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, m->device);
      if (e != cudaSuccess || n < 1)
        return fail_na(GAPGB_ERR_CUDA,
                       std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
      g_sms[m->device] = n;
      g_ptr[m->device] = static_cast<double *>(p);
    }
    scratch = g_ptr[m->device];
    sms = g_sms[m->device];
  }
  // split over sparse points: enough blocks for the GPU, bounded by the scratch
  const int bx = (natoms + kNBM - 1) / kNBM;
  const int kt = (M + kNBK - 1) / kNBK;
  int ns = (2 * sms + bx - 1) / bx;
  if (ns > kt) ns = kt;
  const int ns_fit = (int)(kNoAllocScratch / per_split);
  if (ns > ns_fit) ns = ns_fit;
  if (ns < 1) ns = 1;
  const int klen = ((kt + ns - 1) / ns) * kNBK;
  const int nsp = (M + klen - 1) / klen;
  double *part_e = scratch;
  double *part_d = scratch + (size_t)nsp * natoms;
  const size_t smem = noalloc_smem(D);
  cudaStream_t st = (cudaStream_t)stream;
  k_gpr_noalloc<<<dim3(bx, nsp), 256, smem, st>>>(natoms, M, D, klen, d_G, m->d_mmt, m->d_invth,
                                                   m->d_coeff, part_e, part_d);
  const size_t nd = (size_t)natoms * D;
  k_gpr_noalloc_sum<<<(unsigned)((nd + 255) / 256), 256, 0, st>>>(natoms, D, nsp, part_e, part_d,
                                                                   d_e, d_dedg);
  GAPGB_CUDA_TRY(cudaGetLastError());
  return GAPGB_OK;
}
