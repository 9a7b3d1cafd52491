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
// expansion), so there is no cancellation beyond the reference's own; e_i is
// accumulated in FP64 with the coefficients in FP64 in every form.
//
// T is the arithmetic type, TG the storage type of G and dE/dG (the mixed
// form reads FP32 descriptors and runs the GPR in FP64).
//
// Tiling: a block of 256 threads owns 64 atoms and walks the sparse points in
// tiles of 64 staged in shared memory.  Phase A: thread (ty, tx) forms the
// 4 x 4 kernel values of atoms ty+16a and points tx+16b (8 shared loads per
// 16 difference-square-adds).  Phase B: the same thread accumulates dE/dG of
// atoms ty+16a and descriptor components tx+16b.  Small batches split the
// sparse points over blockIdx.y; a fixed-order reduction sums the partials.
#include <algorithm>
#include <type_traits>

#include "gapgb_internal.h"

namespace gapgb {
namespace {

constexpr int kBM = 64;
constexpr int kBK = 64;

__device__ __forceinline__ double g_exp(double x) { return exp(x); }
__device__ __forceinline__ float g_exp(float x) { return expf(x); }

// One work item: atoms [i0, i0 + 64) of a list of N rows (row i is atom
// rows[i], or atom i when rows is null) against sparse points [kbeg, kend);
// partial results go to e_out[base + i] and dedg_out[(base + i) * D + d].
template <typename T, typename TG, int NB>
__device__ __forceinline__ void gpr_tile(int N, int D, int i0, int kbeg, int kend, size_t base0,
                                         const int *__restrict__ rows, const TG *__restrict__ G,
                                         const T *__restrict__ mmt, const T *__restrict__ invth,
                                         const double *__restrict__ coeff,
                                         const float *__restrict__ coeff32,
                                         double *__restrict__ e_out, T *__restrict__ dedg_out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ld = D + 1;
  T *xs = reinterpret_cast<T *>(smraw);  // [kBM][D+1]
  T *ms = xs + kBM * ld;                 // [kBK][D+1]
  T *ws = ms + kBK * ld;                 // [kBM][kBK+1]
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  for (int q = t; q < kBM * D; q += 256) {
    const int r = q / D, d = q - r * D;
    const int i = i0 + r;
    const size_t a = rows ? (size_t)(i < N ? rows[i] : 0) : (size_t)i;
    xs[r * ld + d] = (i < N) ? (T)G[a * D + d] * invth[d] : (T)0;
  }
  __syncthreads();
  T xr[4][NB];
  T acc[4][NB];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int d = tx + 16 * b;
      xr[a][b] = (d < D) ? xs[(ty + 16 * a) * ld + d] : (T)0;
      acc[a][b] = (T)0;
    }
  // e partial sums: FP64 in the FP64 form; in the FP32 form a compensated
  // FP32 pair (hi + lo), which keeps the FP64 pipe out of the inner loop
  double epart[4] = {0.0, 0.0, 0.0, 0.0};
  float ehi[4] = {0.f, 0.f, 0.f, 0.f}, elo[4] = {0.f, 0.f, 0.f, 0.f};
  constexpr bool kF64 = std::is_same<T, double>::value;
  for (int k0 = kbeg; k0 < kend; k0 += kBK) {
    for (int q = t; q < kBK * D; q += 256) {
      const int r = q / D, d = q - r * D;
      const int k = k0 + r;
      ms[r * ld + d] = (k < kend) ? mmt[(size_t)k * D + d] : (T)0;
    }
    __syncthreads();
    // phase A: 4 x 4 kernel values per thread
    T s[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) s[a][b] = (T)0;
#pragma unroll 4
    for (int d = 0; d < D; ++d) {
      T xv[4], mv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) xv[a] = xs[(ty + 16 * a) * ld + d];
#pragma unroll
      for (int b = 0; b < 4; ++b) mv[b] = ms[(tx + 16 * b) * ld + d];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const T df = xv[a] - mv[b];
          s[a][b] += df * df;
        }
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int k = k0 + tx + 16 * b;
      if (kF64) {
        const double c = (k < kend) ? coeff[k] : 0.0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const T K = g_exp((T)-0.5 * s[a][b]);
          const double w = (double)K * c;
          epart[a] += w;
          ws[(ty + 16 * a) * (kBK + 1) + tx + 16 * b] = (T)w;
        }
      } else {
        const float c = (k < kend) ? coeff32[k] : 0.f;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const float w = (float)g_exp((T)-0.5 * s[a][b]) * c;
          const float t = ehi[a] + w;  // two-sum of (ehi, w)
          const float bb = t - ehi[a];
          elo[a] += (ehi[a] - (t - bb)) + (w - bb);
          ehi[a] = t;
          ws[(ty + 16 * a) * (kBK + 1) + tx + 16 * b] = (T)w;
        }
      }
    }
    __syncthreads();
    // phase B: dE/dG partial sums
    const int kn = min(kBK, kend - k0);
    for (int kk = 0; kk < kn; ++kk) {
      T w[4], mv[NB];
#pragma unroll
      for (int a = 0; a < 4; ++a) w[a] = ws[(ty + 16 * a) * (kBK + 1) + kk];
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        const int d = tx + 16 * b;
        mv[b] = (d < D) ? ms[kk * ld + d] : (T)0;
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < NB; ++b) acc[a][b] += (xr[a][b] - mv[b]) * w[a];
    }
    __syncthreads();
  }
  // e: reduce over the 16 threads (tx) that share an atom row
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    double v = kF64 ? epart[a] : (double)ehi[a] + (double)elo[a];
#pragma unroll
    for (int off = 1; off < 16; off <<= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    epart[a] = v;
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = i0 + ty + 16 * a;
    if (i >= N) continue;
    const size_t base = base0 + i;
    if (tx == 0) e_out[base] = epart[a];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int d = tx + 16 * b;
      if (d < D) dedg_out[base * D + d] = -acc[a][b] * invth[d];
    }
  }
}

template <typename T, typename TG, int NB>
__global__ void __launch_bounds__(256)
    k_gpr(int N, int M, int D, int klen, const TG *__restrict__ G, const T *__restrict__ mmt,
          const T *__restrict__ invth, const double *__restrict__ coeff,
          const float *__restrict__ coeff32,
          double *__restrict__ e_out, T *__restrict__ dedg_out) {
  const int kbeg = blockIdx.y * klen;
  gpr_tile<T, TG, NB>(N, D, blockIdx.x * kBM, kbeg, min(M, kbeg + klen), (size_t)blockIdx.y * N,
                      nullptr, G, mmt, invth, coeff, coeff32, e_out, dedg_out);
}

// Split of a device-counted row list over `nblocks` persistent blocks: enough
// sparse-point splits that the (row tile, split) items fill the blocks.
struct RowSplit {
  int ntiles, nsp, klen;
};
__host__ __device__ inline RowSplit row_split(int count, int M, int nblocks) {
  RowSplit r;
  r.ntiles = (count + kBM - 1) / kBM;
  const int kt = (M + kBK - 1) / kBK;
  int ns = r.ntiles > 0 ? (nblocks + r.ntiles - 1) / r.ntiles : 1;
  ns = ns < 1 ? 1 : (ns > kt ? kt : ns);
  r.klen = ((kt + ns - 1) / ns) * kBK;
  r.nsp = (M + r.klen - 1) / r.klen;
  return r;
}

// The GPR over the atoms listed in rows[0 .. *count): persistent blocks walk
// the (row tile, sparse split) items, so the launch shape is independent of
// the count (CUDA-graph friendly).  Partials: split p of row i at p * count + i.
template <typename T, typename TG, int NB>
__global__ void __launch_bounds__(256)
    k_gpr_rows(const int *__restrict__ count, const int *__restrict__ rows, int M, int D,
               const TG *__restrict__ G, const T *__restrict__ mmt, const T *__restrict__ invth,
               const double *__restrict__ coeff, const float *__restrict__ coeff32,
               double *__restrict__ e_out, T *__restrict__ dedg_out) {
  const int n = *count;
  const RowSplit rs = row_split(n, M, gridDim.x);
  for (int w = blockIdx.x; w < rs.ntiles * rs.nsp; w += gridDim.x) {
    const int tile = w / rs.nsp, p = w - tile * rs.nsp;
    const int kbeg = p * rs.klen;
    __syncthreads();  // the previous item's last reads of the shared tiles
    gpr_tile<T, TG, NB>(n, D, tile * kBM, kbeg, min(M, kbeg + rs.klen), (size_t)p * n, rows, G,
                        mmt, invth, coeff, coeff32, e_out, dedg_out);
  }
}

template <typename T, typename TG>
__global__ void k_gpr_reduce_rows(int cap, int D, int M, int nblocks, const int *__restrict__ count,
                                  const int *__restrict__ rows, const double *__restrict__ e_part,
                                  const T *__restrict__ dedg_part, double *__restrict__ e,
                                  TG *__restrict__ dedg) {
  const int n = *count;
  const RowSplit rs = row_split(n, M, nblocks);
  const size_t nd = (size_t)n * D;
  // grid-stride over the listed rows only (the grid does not depend on n)
  for (size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x; tid < nd;
       tid += (size_t)gridDim.x * blockDim.x) {
    T s = (T)0;
    for (int p = 0; p < rs.nsp; ++p) s += dedg_part[(size_t)p * nd + tid];
    const size_t i = tid / D;
    dedg[(size_t)rows[i] * D + (tid - i * D)] = (TG)s;
    if (tid - i * D == 0) {
      double se = 0.0;
      for (int p = 0; p < rs.nsp; ++p) se += e_part[(size_t)p * n + i];
      e[rows[i]] = se;
    }
  }
  (void)cap;
}

template <typename T, typename TG>
__global__ void k_gpr_reduce(int N, int D, int nsplit, const double *__restrict__ e_part,
                             const T *__restrict__ dedg_part, double *__restrict__ e,
                             TG *__restrict__ dedg) {
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t nd = (size_t)N * D;
  if (tid < nd) {
    T s = (T)0;
    for (int p = 0; p < nsplit; ++p) s += dedg_part[(size_t)p * nd + tid];
    dedg[tid] = (TG)s;
  }
  if (tid < (size_t)N) {
    double s = 0.0;
    for (int p = 0; p < nsplit; ++p) s += e_part[(size_t)p * N + tid];
    e[tid] = s;
  }
}

}  // namespace

int gpr_nsplit(int N, int M) {
  const int sms = device_sms();
  const int bx = (N + kBM - 1) / kBM;
  const int kt = (M + kBK - 1) / kBK;
  int ns = (2 * sms + bx - 1) / bx;
  if (ns < 1) ns = 1;
  if (ns > kt) ns = kt;
  return ns;
}

size_t gpr_scratch_bytes(int N, int M, int D, size_t elem) {
  // partial e and dE/dG of every split (one split still stages here so that
  // the reduction also casts to the storage type)
  const int ns = gpr_nsplit(N, M);
  return (size_t)ns * N * sizeof(double) + (size_t)ns * N * D * elem;
}

template <typename T, typename TG>
void launch_gpr(const gapgb_model *m, Workspace &ws, int N, cudaStream_t st) {
  const int M = m->host.M, D = m->host.D;
  const int ns = gpr_nsplit(N, M);
  const int kt = (M + kBK - 1) / kBK;
  const int klen = ((kt + ns - 1) / ns) * kBK;
  const int nsp = (M + klen - 1) / klen;
  const size_t smem = ((size_t)(kBM + kBK) * (D + 1) + (size_t)kBM * (kBK + 1)) * sizeof(T);
  constexpr bool f64 = std::is_same<T, double>::value;
  const T *mmt = f64 ? (const T *)m->d_mmt : (const T *)m->d_mmt32;
  const T *invth = f64 ? (const T *)m->d_invth : (const T *)m->d_invth32;
  dim3 grid((N + kBM - 1) / kBM, nsp);
  double *e_part = reinterpret_cast<double *>(ws.gpr_scratch);
  T *d_part = reinterpret_cast<T *>(e_part + (size_t)nsp * N);
  const TG *G = (const TG *)ws.G;
  auto run = [&](auto fn) {
    kernel_smem((const void *)fn, (int)smem);
    fn<<<grid, 256, smem, st>>>(N, M, D, klen, G, mmt, invth, m->d_coeff, m->d_coeff32, e_part,
                                d_part);
  };
  if (D <= 64) run(k_gpr<T, TG, 4>);
  else run(k_gpr<T, TG, 8>);
  const size_t nd = (size_t)N * D;
  k_gpr_reduce<T, TG><<<(unsigned)((nd + 255) / 256), 256, 0, st>>>(N, D, nsp, e_part, d_part,
                                                                     ws.e, (TG *)ws.dedg);
}

constexpr int kRowBlocksPerSm = 2;

int gpr_rows_blocks() {
  const int sms = device_sms();
  return kRowBlocksPerSm * sms;
}

size_t gpr_rows_scratch_bytes(int cap, int D) {
  // rows of partials: nsp * count <= max(cap, (nblocks + ntiles) * 64)
  const size_t rows = (size_t)cap + (size_t)(gpr_rows_blocks() + 1) * kBM + (size_t)cap / kBM + kBM;
  return rows * sizeof(double) * (size_t)(D + 1);
}

// FP64 GPR (FP32 descriptors, FP32 dE/dG out: the mixed form) of the atoms
// d_rows[0 .. *d_count), d_count <= cap, written into ws.e / ws.dedg at
// those atoms.  The scratch holds gpr_rows_scratch_bytes(cap, D).
void launch_gpr_rows(const gapgb_model *m, Workspace &ws, int cap, const int *d_rows,
                     const int *d_count, void *scratch, cudaStream_t st) {
  const int M = m->host.M, D = m->host.D;
  const int nb = gpr_rows_blocks();
  const size_t smem = ((size_t)(kBM + kBK) * (D + 1) + (size_t)kBM * (kBK + 1)) * sizeof(double);
  const size_t prow = gpr_rows_scratch_bytes(cap, D) / (sizeof(double) * (D + 1));
  double *e_part = reinterpret_cast<double *>(scratch);
  double *d_part = e_part + prow;
  const float *G = (const float *)ws.G;
  auto run = [&](auto fn) {
    kernel_smem((const void *)fn, (int)smem);
    fn<<<nb, 256, smem, st>>>(d_count, d_rows, M, D, G, m->d_mmt, m->d_invth, m->d_coeff,
                              m->d_coeff32, e_part, d_part);
  };
  if (D <= 64) run(k_gpr_rows<double, float, 4>);
  else run(k_gpr_rows<double, float, 8>);
  const size_t nd = (size_t)cap * D;
  const unsigned rb = (unsigned)std::min<size_t>((nd + 255) / 256, (size_t)nb * 4);
  k_gpr_reduce_rows<double, float><<<rb > 0 ? rb : 1, 256, 0, st>>>(
      cap, D, M, nb, d_count, d_rows, e_part, d_part, ws.e, (float *)ws.dedg);
}

template void launch_gpr<double, double>(const gapgb_model *, Workspace &, int, cudaStream_t);
template void launch_gpr<float, float>(const gapgb_model *, Workspace &, int, cudaStream_t);
template void launch_gpr<double, float>(const gapgb_model *, Workspace &, int, cudaStream_t);

}  // namespace gapgb
