// variance.cu - predictive variance of the sparse GPR.
//
// The commented-out block of FGAP_CALC (gappy/libgap/gap_calc.f90:206-210):
//   covf_i   = delta - k_i^T qmm k_i,   k_i = ckm(i, :) from GET_COV (:268-288)
//   VARIANCE = sum_i covf_i / na
// with delta = 1 (gap_calc.f90:8) and qmm an M x M matrix the caller attaches
// (FGAP_READ zero-fills it, :361, so the reference always returns 0).
//
// Batched over atoms this is one N x M x M contraction:
//   V = K qmm^T  (V_im = sum_n K_in qmm_mn),   covf_i = delta - sum_m K_im V_im.
// Two forms:
//  - FP64: K in FP64 (row-major chunk of atoms), a register-tiled FP64 GEMM
//    whose epilogue takes the row dot with K;
//  - tensor cores: K in FP32 from FP32 descriptors, split into BF16 hi + lo
//    and written as pre-arranged operand tiles; qmm split the same way once
//    per attach.  One CTA owns 128 atoms x 256 sparse points of V:
//    tcgen05.mma (M=128, N=256, K=16) accumulates Kh.Qh + Kh.Ql + Kl.Qh in
//    TMEM over the whole contraction while a 4-stage ring of 1-D bulk copies
//    streams 32-wide chunks of both operands; the epilogue reads V back with
//    tcgen05.ld and dots it with the CTA's own K columns.
// Per-row partial dots are written per column tile and summed in a fixed
// order in FP64, so both forms are deterministic.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "gapgb_internal.h"
#include "tc_util.cuh"

namespace gapgb {
namespace {

using namespace tc;

constexpr double kDelta = 1.0;  // gap_calc.f90:8

// ---------------------------------------------------------------- FP64 form
constexpr int kT64 = 64;        // GEMM tile: 64 atoms x 64 sparse points
constexpr int kKC64 = 16;       // contraction chunk of the FP64 GEMM
constexpr int kKm64Rows = 32;   // K-matrix kernel: 32 atoms x 64 sparse points
constexpr int kDChunk = 32;     // descriptor chunk staged in shared memory

// K[r][k] = delta exp(-1/2 sum_d (x_id / theta_d - m_kd / theta_d)^2) for the
// chunk's rows r (atoms row0 + r); zero for padded rows and columns
template <typename TG>
__global__ void __launch_bounds__(256)
    k_var_kmat64(int row0, int N, int M, int Mp, int D, const TG *__restrict__ G,
                 const double *__restrict__ invth, const double *__restrict__ mmt,
                 double *__restrict__ K) {
  __shared__ double xs[kKm64Rows][kDChunk + 1];
  __shared__ double ms[kT64][kDChunk + 1];
  const int tid = threadIdx.x, tx = tid & 63, ty = tid >> 6;
  const int rb = blockIdx.y * kKm64Rows, kb = blockIdx.x * kT64;
  double acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = 0.0;
  for (int d0 = 0; d0 < D; d0 += kDChunk) {
    for (int e = tid; e < kKm64Rows * kDChunk; e += 256) {
      const int r = e / kDChunk, d = d0 + e % kDChunk, i = row0 + rb + r;
      xs[r][e % kDChunk] = (i < N && d < D) ? (double)G[(size_t)i * D + d] * invth[d] : 0.0;
    }
    for (int e = tid; e < kT64 * kDChunk; e += 256) {
      const int k = kb + e / kDChunk, d = d0 + e % kDChunk;
      ms[e / kDChunk][e % kDChunk] = (k < M && d < D) ? mmt[(size_t)k * D + d] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int d = 0; d < kDChunk; ++d) {
      const double mv = ms[tx][d];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const double t = xs[ty + 4 * q][d] - mv;
        acc[q] += t * t;
      }
    }
    __syncthreads();
  }
  const int k = kb + tx;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int r = rb + ty + 4 * q;
    const bool live = row0 + r < N && k < M;
    K[(size_t)r * Mp + k] = live ? kDelta * exp(-0.5 * acc[q]) : 0.0;
  }
}

// part[r][blockIdx.x] = sum_{m in tile} K_rm (sum_n K_rn Q_mn)
__global__ void __launch_bounds__(256)
    k_var_gemm64(int rows, int Mp, const double *__restrict__ K, const double *__restrict__ Q,
                 double *__restrict__ part) {
  __shared__ double As[kKC64][kT64 + 1];
  __shared__ double Bs[kKC64][kT64 + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int rb = blockIdx.y * kT64, cb = blockIdx.x * kT64;
  const int nT = gridDim.x;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int n0 = 0; n0 < Mp; n0 += kKC64) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = tid + 256 * q, r = e / kKC64, kk = e % kKC64;
      As[kk][r] = K[(size_t)(rb + r) * Mp + n0 + kk];
      Bs[kk][r] = Q[(size_t)(cb + r) * Mp + n0 + kk];
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKC64; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][ty * 4 + u];
        b[u] = Bs[kk][tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int r = rb + ty * 4 + u;
    const double *kr = K + (size_t)r * Mp + cb + tx * 4;
    double d = 0.0;
#pragma unroll
    for (int v = 0; v < 4; ++v) d = fma(acc[u][v], kr[v], d);
    // the 16 lanes of one row sit in one half-warp: fixed-order tree sum
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) d += __shfl_xor_sync(0xffffffffu, d, off);
    if (tx == 0 && r < rows) part[(size_t)r * nT + blockIdx.x] = d;
  }
}

// covf = delta - sum over the column tiles (ascending), FP64
__global__ void k_var_finish(int rows, int row0, int nT, const double *__restrict__ part,
                             double *__restrict__ covf) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double s = 0.0;
  for (int t = 0; t < nT; ++t) s += part[(size_t)r * nT + t];
  covf[row0 + r] = kDelta - s;
}

// VARIANCE of each structure: the mean of its atoms' covf (fixed-order tree)
__global__ void __launch_bounds__(128)
    k_var_struct(const int *__restrict__ atom_off, const double *__restrict__ covf,
                 double *__restrict__ var) {
  __shared__ double red[128];
  const int s = blockIdx.x, a0 = atom_off[s], a1 = atom_off[s + 1];
  double acc = 0.0;
  for (int i = a0 + threadIdx.x; i < a1; i += 128) acc += covf[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) var[s] = a1 > a0 ? red[0] / (double)(a1 - a0) : 0.0;
}

// ------------------------------------------------------- tensor-core form
constexpr int kVRows = 128;  // atoms per CTA (UMMA M)
constexpr int kVN = 256;     // sparse points of V per CTA (UMMA N)
constexpr int kVK = 32;      // contraction chunk per pipeline stage
constexpr int kVStages = 4;
constexpr int kVKHalf = kVRows * kVK * 2;   // 128 x 32 bf16: 8 KB
constexpr int kVQHalf = kVN * kVK * 2;      // 256 x 32 bf16: 16 KB
constexpr int kVKBlk = 2 * kVKHalf;         // K image block (hi, lo)
constexpr int kVQBlk = 2 * kVQHalf;         // qmm image block (hi, lo)
constexpr int kVStage = kVKBlk + kVQBlk;    // 48 KB
constexpr int kVOffBar = kVStages * kVStage;
constexpr int kVOffEp = kVOffBar + 128;     // partial dots of the second column half
constexpr int kVSmem = kVOffEp + kVRows * 8 + 1024;
constexpr int kVThreads = 256;
constexpr int kKimgDC = 32;                 // descriptor chunk of the K-image kernel

// K image: block (atom tile a, chunk c) = 128 rows x 32 sparse points, hi
// then lo, no-swizzle K-major (k = sparse point index within the chunk)
// Descriptors centred on the sparse points' mean mu before the FP32
// differences (x'' - mu formed in FP64 and rounded once; m'' - mu stored),
// so the rounding is relative to |x'' - m''|-sized values, not to |x''|:
// xc[i][d] = G_id / theta_d - mu_d for the atoms of one chunk
template <typename TG>
__global__ void k_var_center(int row0, int rows, int D, const TG *__restrict__ G,
                             const double *__restrict__ invth, const double *__restrict__ mu,
                             float *__restrict__ xc) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)rows * D) return;
  const int d = (int)(e % D);
  xc[e] = (float)((double)G[(size_t)row0 * D + e] * invth[d] - mu[d]);
}

__global__ void __launch_bounds__(256)
    k_var_kimg(int rows, int M, int D, int nch, const float *__restrict__ xc,
               const float *__restrict__ mc, unsigned char *__restrict__ img) {
  __shared__ __align__(16) float xs[kKimgDC][kVRows + 4];
  __shared__ __align__(16) float ms[kKimgDC][kVK + 4];
  const int tid = threadIdx.x;
  const int c = blockIdx.x, a = blockIdx.y;
  const int r0 = (tid >> 2) * 2, k0 = (tid & 3) * 8;
  float acc[2][8];
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int u = 0; u < 8; ++u) acc[q][u] = 0.f;
  for (int d0 = 0; d0 < D; d0 += kKimgDC) {
    for (int e = tid; e < kVRows * kKimgDC; e += 256) {
      const int r = e / kKimgDC, dd = e % kKimgDC, d = d0 + dd;
      const int i = a * kVRows + r;
      xs[dd][r] = (i < rows && d < D) ? xc[(size_t)i * D + d] : 0.f;
    }
    for (int e = tid; e < kVK * kKimgDC; e += 256) {
      const int kk = e / kKimgDC, dd = e % kKimgDC, d = d0 + dd, k = c * kVK + kk;
      ms[dd][kk] = (k < M && d < D) ? mc[(size_t)k * D + d] : 0.f;
    }
    __syncthreads();
#pragma unroll 4
    for (int dd = 0; dd < kKimgDC; ++dd) {
      const float2 x = *reinterpret_cast<const float2 *>(&xs[dd][r0]);
      const float4 m0 = *reinterpret_cast<const float4 *>(&ms[dd][k0]);
      const float4 m1 = *reinterpret_cast<const float4 *>(&ms[dd][k0 + 4]);
      const float mv[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const float t0 = x.x - mv[u], t1 = x.y - mv[u];
        acc[0][u] = fmaf(t0, t0, acc[0][u]);
        acc[1][u] = fmaf(t1, t1, acc[1][u]);
      }
    }
    __syncthreads();
  }
  unsigned char *blk = img + ((size_t)a * nch + c) * kVKBlk;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int r = r0 + q, i = a * kVRows + r;
    uint32_t hp[4], lp[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      float w[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int k = c * kVK + k0 + 2 * h + u;
        w[u] = (i < rows && k < M) ? (float)kDelta * expf(-0.5f * acc[q][2 * h + u]) : 0.f;
      }
      const __nv_bfloat162 hi = __floats2bfloat162_rn(w[0], w[1]);
      const float2 hf = __bfloat1622float2(hi);
      hp[h] = *reinterpret_cast<const uint32_t *>(&hi);
      lp[h] = pack_bf16(w[0] - hf.x, w[1] - hf.y);
    }
    const int off = kmajor_off(r, k0, kVK / 8);
    *reinterpret_cast<uint4 *>(blk + off) = make_uint4(hp[0], hp[1], hp[2], hp[3]);
    *reinterpret_cast<uint4 *>(blk + kVKHalf + off) = make_uint4(lp[0], lp[1], lp[2], lp[3]);
  }
}

__device__ __forceinline__ float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }

__global__ void __launch_bounds__(kVThreads, 1)
    k_var_tc(int nch, int rows, const unsigned char *__restrict__ kimg,
             const unsigned char *__restrict__ qimg, double *__restrict__ part,
             int *__restrict__ flags) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>(
      ((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, half = warp >> 2;
  const int t = blockIdx.x, a = blockIdx.y, nT = gridDim.x;
  const uint32_t s_base = smem_u32(sm);
  const uint32_t bar_full = s_base + kVOffBar;            // kVStages barriers
  const uint32_t bar_empty = bar_full + 8 * kVStages;     // kVStages barriers
  const uint32_t bar_done = bar_empty + 8 * kVStages;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + kVOffBar + 8 * (2 * kVStages + 1));
  int *abort_flag = reinterpret_cast<int *>(sm + kVOffBar + 8 * (2 * kVStages + 1) + 8);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kVStages; ++s) {
      mbar_init(bar_full + 8 * s, 1);
      mbar_init(bar_empty + 8 * s, 1);
    }
    mbar_init(bar_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const unsigned char *kbase = kimg + (size_t)a * nch * kVKBlk;
  const unsigned char *qbase = qimg + (size_t)t * nch * kVQBlk;
  if (tid == 0) {
    const uint32_t idesc = instr_desc(kVRows, kVN);
    int loads[kVStages] = {0, 0, 0, 0};  // copies issued into each stage
    unsigned pend = 0;                   // stages with a copy not yet waited for
    bool ok = true;
    auto load = [&](int c, int s) {
      const uint32_t dst = s_base + s * kVStage;
      mbar_expect_tx(bar_full + 8 * s, kVStage);
      bulk_g2s(dst, kbase + (size_t)c * kVKBlk, kVKBlk, bar_full + 8 * s);
      bulk_g2s(dst + kVKBlk, qbase + (size_t)c * kVQBlk, kVQBlk, bar_full + 8 * s);
      ++loads[s];
      pend |= 1u << s;
    };
    for (int c = 0; c < kVStages - 1 && c < nch; ++c) load(c, c);
    for (int c = 0; c < nch && ok; ++c) {
      const int s = c % kVStages;
      ok = mbar_wait(bar_full + 8 * s, (uint32_t)((c / kVStages) & 1), flags);
      if (!ok) break;
      pend &= ~(1u << s);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t st = s_base + s * kVStage;
      const uint32_t a_off[3] = {0, 0, (uint32_t)kVKHalf};
      const uint32_t b_off[3] = {(uint32_t)kVKBlk, (uint32_t)(kVKBlk + kVQHalf),
                                 (uint32_t)kVKBlk};
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int kk = 0; kk < kVK / 16; ++kk) {
          const uint64_t ad = smem_desc(st + a_off[p] + kk * 256, 128, (kVK / 8) * 128);
          const uint64_t bd = smem_desc(st + b_off[p] + kk * 256, 128, (kVK / 8) * 128);
          umma(tmem, ad, bd, idesc, (c > 0 || p > 0 || kk > 0) ? 1u : 0u);
        }
      umma_commit(bar_empty + 8 * s);
      // refill the stage of chunk c - 1 (its MMAs finish before chunk c's run)
      const int nxt = c + kVStages - 1;
      if (nxt < nch) {
        const int sn = nxt % kVStages;
        if (c >= 1) {
          ok = mbar_wait(bar_empty + 8 * sn, (uint32_t)(((c - 1) / kVStages) & 1), flags);
          if (!ok) break;
        }
        load(nxt, sn);
      }
    }
    if (!ok) {
      // a wait gave up: one more bounded wait for every copy still in flight
      for (int s = 0; s < kVStages; ++s)
        if (pend & (1u << s)) mbar_wait(bar_full + 8 * s, (uint32_t)((loads[s] - 1) & 1), flags);
    }
    umma_commit(bar_done);  // completes when every MMA issued above has
    if (!mbar_wait(bar_done, 0, flags)) ok = false;
    *abort_flag = ok ? 0 : 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const int row = quad * 32 + lane;
  if (!*abort_flag) {
    const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
    float dot = 0.f;
#pragma unroll 1
    for (int cb = 0; cb < 4; ++cb) {
      const int col0 = half * 128 + cb * 32;  // within this CTA's 256 columns
      float v[32];
      tmem_ld32(tmem + lane_base + col0, v);
      const int c = (t * kVN + col0) / kVK;   // the K-image chunk of these columns
      const unsigned char *blk = kbase + (size_t)c * kVKBlk;
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        const int off = kmajor_off(row, g * 8, kVK / 8);
        const uint4 h = *reinterpret_cast<const uint4 *>(blk + off);
        const uint4 l = *reinterpret_cast<const uint4 *>(blk + kVKHalf + off);
        const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, lw[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          dot = fmaf(v[g * 8 + 2 * e], bf16_lo(hw[e]) + bf16_lo(lw[e]), dot);
          dot = fmaf(v[g * 8 + 2 * e + 1], bf16_hi(hw[e]) + bf16_hi(lw[e]), dot);
        }
      }
    }
    double *ep = reinterpret_cast<double *>(sm + kVOffEp);
    if (half == 1) ep[row] = (double)dot;
    __syncthreads();
    const int r = a * kVRows + row;
    if (half == 0 && r < rows) part[(size_t)r * nT + t] = (double)dot + ep[row];
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem) : "memory");
}

// host-side bf16 (round to nearest even)
uint16_t to_bf16(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
float from_bf16(uint16_t b) {
  const uint32_t u = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

int padded_m(int M) { return (M + kVN - 1) / kVN * kVN; }

gapgb_status ensure_buf(void **p, size_t *have, size_t need) {
  if (*have >= need) return GAPGB_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *have = 0;
  if (cudaMalloc(p, need) != cudaSuccess) {
    set_last_error("cudaMalloc of " + std::to_string(need) + " bytes for the variance failed");
    return GAPGB_ERR_CUDA;
  }
  *have = need;
  return GAPGB_OK;
}

gapgb_status build_q64(gapgb_model *m) {
  VarState &v = m->var;
  if (v.d_q64) return GAPGB_OK;
  const int M = m->host.M, Mp = padded_m(M);
  std::vector<double> q((size_t)Mp * Mp, 0.0);
  for (int r = 0; r < M; ++r)
    std::memcpy(q.data() + (size_t)r * Mp, v.qmm.data() + (size_t)r * M, sizeof(double) * M);
  GAPGB_CUDA_TRY(cudaMalloc(&v.d_q64, sizeof(double) * q.size()));
  GAPGB_CUDA_TRY(cudaMemcpy(v.d_q64, q.data(), sizeof(double) * q.size(), cudaMemcpyHostToDevice));
  return GAPGB_OK;
}

// qmm image: block (column tile t of 256 rows of qmm, chunk c of 32) = hi
// then lo, no-swizzle K-major (B operand row = qmm row m, K index = n)
gapgb_status build_qimg(gapgb_model *m) {
  VarState &v = m->var;
  if (v.d_qimg) return GAPGB_OK;
  const int M = m->host.M, D = m->host.D, Mp = padded_m(M), nch = Mp / kVK, nT = Mp / kVN;
  if (!v.d_mc32) {
    // sparse points scaled by 1/theta and centred on their mean (FP64, then FP32)
    const HostModel &h = m->host;
    std::vector<double> mu(D, 0.0);
    for (int k = 0; k < M; ++k)
      for (int d = 0; d < D; ++d) mu[d] += h.mm[(size_t)k * D + d] / h.theta[d];
    for (int d = 0; d < D; ++d) mu[d] /= M;
    std::vector<float> mc((size_t)M * D);
    for (int k = 0; k < M; ++k)
      for (int d = 0; d < D; ++d)
        mc[(size_t)k * D + d] = (float)(h.mm[(size_t)k * D + d] / h.theta[d] - mu[d]);
    GAPGB_CUDA_TRY(cudaMalloc(&v.d_mu64, sizeof(double) * D));
    GAPGB_CUDA_TRY(cudaMemcpy(v.d_mu64, mu.data(), sizeof(double) * D, cudaMemcpyHostToDevice));
    GAPGB_CUDA_TRY(cudaMalloc(&v.d_mc32, sizeof(float) * mc.size()));
    GAPGB_CUDA_TRY(cudaMemcpy(v.d_mc32, mc.data(), sizeof(float) * mc.size(), cudaMemcpyHostToDevice));
  }
  std::vector<unsigned char> img((size_t)nT * nch * kVQBlk, 0);
  for (int mrow = 0; mrow < M; ++mrow) {
    const int t = mrow / kVN, r = mrow % kVN;
    for (int n = 0; n < M; ++n) {
      const int c = n / kVK, k = n % kVK;
      const float x = (float)v.qmm[(size_t)mrow * M + n];
      const uint16_t hi = to_bf16(x);
      const uint16_t lo = to_bf16(x - from_bf16(hi));
      unsigned char *blk = img.data() + ((size_t)t * nch + c) * kVQBlk;
      const int off = kmajor_off(r, k, kVK / 8);
      std::memcpy(blk + off, &hi, 2);
      std::memcpy(blk + kVQHalf + off, &lo, 2);
    }
  }
  GAPGB_CUDA_TRY(cudaMalloc(&v.d_qimg, img.size()));
  GAPGB_CUDA_TRY(cudaMemcpy(v.d_qimg, img.data(), img.size(), cudaMemcpyHostToDevice));
  return GAPGB_OK;
}

}  // namespace

void variance_free(VarState &v) {
  if (v.d_mu64) cudaFree(v.d_mu64);
  if (v.d_mc32) cudaFree(v.d_mc32);
  v.d_mu64 = nullptr;
  v.d_mc32 = nullptr;
  if (v.d_q64) cudaFree(v.d_q64);
  if (v.d_qimg) cudaFree(v.d_qimg);
  if (v.kbuf) cudaFree(v.kbuf);
  if (v.part) cudaFree(v.part);
  if (v.xc) cudaFree(v.xc);
  v.xc = nullptr;
  v.xc_bytes = 0;
  if (v.covf) cudaFree(v.covf);
  if (v.var) cudaFree(v.var);
  v.d_q64 = nullptr;
  v.d_qimg = nullptr;
  v.kbuf = v.part = v.covf = v.var = nullptr;
  v.kbuf_bytes = v.part_bytes = v.covf_bytes = v.var_bytes = 0;
}

gapgb_status variance_set_qmm(gapgb_model *m, const double *qmm) {
  VarState &v = m->var;
  if (v.d_q64) cudaFree(v.d_q64);
  if (v.d_qimg) cudaFree(v.d_qimg);
  v.d_q64 = nullptr;
  v.d_qimg = nullptr;
  if (!qmm) {
    v.qmm.clear();
    return GAPGB_OK;
  }
  const size_t M = (size_t)m->host.M;
  v.qmm.assign(qmm, qmm + M * M);
  return GAPGB_OK;
}

bool variance_fp64_form(const gapgb_model *m) {
  return m->precision == GAPGB_PREC_FP64 || m->precision == GAPGB_PREC_MIXED;
}

size_t variance_tc_smem_bytes() { return kVSmem; }

gapgb_status variance_enqueue(gapgb_model *m, int S, int N, const int *d_atom_off, const void *G,
                              bool g64, cudaStream_t st) {
  VarState &v = m->var;
  if (v.qmm.empty()) {
    set_last_error("no qmm attached (gapgb_model_set_qmm)");
    return GAPGB_ERR_ARG;
  }
  const int M = m->host.M, D = m->host.D, Mp = padded_m(M);
  gapgb_status s = ensure_buf(&v.covf, &v.covf_bytes, sizeof(double) * (size_t)(N > 0 ? N : 1));
  if (s) return s;
  s = ensure_buf(&v.var, &v.var_bytes, sizeof(double) * (size_t)(S > 0 ? S : 1));
  if (s) return s;
  if (variance_fp64_form(m)) {
    s = build_q64(m);
    if (s) return s;
    const int chunk = 8192;  // atoms per K chunk (Mp * 64 KB of FP64 K)
    const int nT = Mp / kT64;
    s = ensure_buf(&v.kbuf, &v.kbuf_bytes, sizeof(double) * (size_t)chunk * Mp);
    if (s) return s;
    s = ensure_buf(&v.part, &v.part_bytes, sizeof(double) * (size_t)chunk * nT);
    if (s) return s;
    for (int r0 = 0; r0 < N; r0 += chunk) {
      const int rows = std::min(chunk, N - r0);
      const int rpad = (rows + kT64 - 1) / kT64 * kT64;
      const dim3 gk(Mp / kT64, rpad / kKm64Rows), gg(nT, rpad / kT64);
      if (g64)
        k_var_kmat64<double><<<gk, 256, 0, st>>>(r0, N, M, Mp, D, (const double *)G, m->d_invth,
                                                 m->d_mmt, (double *)v.kbuf);
      else
        k_var_kmat64<float><<<gk, 256, 0, st>>>(r0, N, M, Mp, D, (const float *)G, m->d_invth,
                                                m->d_mmt, (double *)v.kbuf);
      k_var_gemm64<<<gg, 256, 0, st>>>(rows, Mp, (const double *)v.kbuf, v.d_q64,
                                        (double *)v.part);
      k_var_finish<<<(rows + 127) / 128, 128, 0, st>>>(rows, r0, nT, (const double *)v.part,
                                                        (double *)v.covf);
    }
  } else {
    s = build_qimg(m);
    if (s) return s;
    GAPGB_CUDA_TRY(cudaFuncSetAttribute(k_var_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kVSmem));
    const int chunk = 65536;  // atoms per K image (Mp * 256 KB)
    const int nch = Mp / kVK, nT = Mp / kVN;
    s = ensure_buf(&v.kbuf, &v.kbuf_bytes, (size_t)(chunk / kVRows) * nch * kVKBlk);
    if (s) return s;
    s = ensure_buf(&v.part, &v.part_bytes, sizeof(double) * (size_t)chunk * nT);
    if (s) return s;
    s = ensure_buf(&v.xc, &v.xc_bytes, sizeof(float) * (size_t)chunk * D);
    if (s) return s;
    for (int r0 = 0; r0 < N; r0 += chunk) {
      const int rows = std::min(chunk, N - r0);
      const int nA = (rows + kVRows - 1) / kVRows;
      const unsigned nb = (unsigned)(((size_t)rows * D + 255) / 256);
      if (g64)
        k_var_center<double><<<nb, 256, 0, st>>>(r0, rows, D, (const double *)G, m->d_invth,
                                                 v.d_mu64, (float *)v.xc);
      else
        k_var_center<float><<<nb, 256, 0, st>>>(r0, rows, D, (const float *)G, m->d_invth,
                                                v.d_mu64, (float *)v.xc);
      k_var_kimg<<<dim3(nch, nA), 256, 0, st>>>(rows, M, D, nch, (const float *)v.xc, v.d_mc32,
                                                (unsigned char *)v.kbuf);
      k_var_tc<<<dim3(nT, nA), kVThreads, kVSmem, st>>>(nch, rows, (const unsigned char *)v.kbuf,
                                                          v.d_qimg, (double *)v.part,
                                                          m->ws.d_flags);
      k_var_finish<<<(rows + 127) / 128, 128, 0, st>>>(rows, r0, nT, (const double *)v.part,
                                                        (double *)v.covf);
    }
  }
  if (S > 0)
    k_var_struct<<<S, 128, 0, st>>>(d_atom_off, (const double *)v.covf, (double *)v.var);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(std::string("variance kernel launch: ") + cudaGetErrorString(e));
    return GAPGB_ERR_CUDA;
  }
  return GAPGB_OK;
}

}  // namespace gapgb
