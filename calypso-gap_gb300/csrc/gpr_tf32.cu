// gpr_tf32.cu - the sparse-GPR contraction on the tensor cores in TF32.
//
// The quantities of gpr.cu / gpr_tc.cu (GET_COV and the energy / dE/dG loops
// of FGAP_CALC, gappy/libgap/gap_calc.f90:143-166, 268-288) with single-term
// TF32 products and FP32 accumulation (tcgen05.mma kind::tf32):
//   x~, m~  = x'' and m'' rounded to TF32 (nearest)
//   s_ik    = |x~_i|^2 + |m~_k|^2 - 2 x~_i . m~_k      (GEMM1, K = D)
//           = |x~_i - m~_k|^2 up to FP32 rounding, so a close pair keeps a
//             small distance error (the rounding of x and m enters as
//             (x - m).(dx - dm), not as |x| |m| 2^-11)
//   w_ik    = c_k exp(-s_ik / 2),  e_i = sum_k w_ik (compensated FP32, Kahan)
//   (W M~)  GEMM2 with W rounded to TF32, K = M
//   dE/dG_id = -(1/theta_d) (x''_id e_i - (W M~)_id)
// The same CTA structure as the split-BF16 kernel: 128 atoms per CTA, tiles of
// 64 sparse points whose GEMM1 half (m~, b2, c) and GEMM2 half (m~^T) load
// under the other half's compute; 8 warps share the epilogue; two CTAs per SM.  Operands
// are K-major, no swizzle, 32-bit elements: core matrices of 8 rows x 4
// elements (16 B), K-adjacent cores 128 B apart, 8-row groups (K/4) * 128 B
// apart; one MMA consumes K = 8.  Every mbarrier wait is bounded.
#include <cstring>
#include <vector>

#include "gapgb_internal.h"
#include "tc_util.cuh"

namespace gapgb {
namespace {

using namespace tc;

constexpr int kRows = 128;  // atoms per CTA (UMMA M)
constexpr int kTK = 64;     // sparse points per tile
constexpr int kDP = 64;     // padded descriptor length
constexpr int kXBytes = kRows * kDP * 4;   // 32 KB
constexpr int kMBytes = kTK * kDP * 4;     // 16 KB (m~ and m~^T each)
constexpr int kWBytes = kRows * kTK * 4;   // 32 KB
constexpr int kMncBytes = 2 * kTK * 4;     // b2 and c of one tile
constexpr int kImgTile = 2 * kMBytes + kMncBytes;
// shared memory map (from the 1024-aligned base)
constexpr int kOffX = 0;
constexpr int kOffM = kOffX + kXBytes;
constexpr int kOffMT = kOffM + kMBytes;
constexpr int kOffMnc = kOffMT + kMBytes;   // two tiles' vectors
constexpr int kOffW = kOffMnc + 2 * kMncBytes;
constexpr int kOffBar = kOffW + kWBytes;
constexpr int kOffEp = kOffBar + 64;
constexpr int kSmem = kOffEp + kRows * 8 + 1024;  // about 99 KB: two CTAs per SM
constexpr int kThreads = 256;
constexpr int kTmemCols = 128;  // C1 (kTK columns) and C2 (kDP columns)

__host__ __device__ __forceinline__ int kmajor32(int r, int k, int kcores) {
  return (r & 7) * 16 + (r >> 3) * (kcores * 128) + (k & 3) * 4 + (k >> 2) * 128;
}

// instruction descriptor, kind::tf32: TF32 x TF32 -> F32, both K-major
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// FP32 -> TF32 (round to nearest, ties away) as a 32-bit pattern
__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__global__ void __launch_bounds__(kThreads, 2)
    k_gpr_tf32(int N, int ntiles, const unsigned char *__restrict__ img_model,
               const unsigned char *__restrict__ img_atoms, const float *__restrict__ xs,
               const float *__restrict__ xn, const float *__restrict__ invth, int D,
               double *__restrict__ e_out, float *__restrict__ dedg, int *__restrict__ flags) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sm =
      reinterpret_cast<unsigned char *>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, half = warp >> 2;
  const uint32_t s_base = smem_u32(sm);
  const uint32_t bar_a = s_base + kOffBar, bar_g1 = bar_a + 8, bar_g2 = bar_a + 16,
                 bar_b = bar_a + 24;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + kOffBar + 32);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "n"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(bar_a, 1);
    mbar_init(bar_g1, 1);
    mbar_init(bar_g2, 1);
    mbar_init(bar_b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t tC1 = tmem, tC2 = tmem + kTK;
  const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
  const int row = quad * 32 + lane;
  const int i = blockIdx.x * kRows + row;
  const float xnorm = (i < N) ? xn[i] : 0.f;
  // w = c 2^(log2e v + a2_i + b2_k) (the image stores b2_k = -log2e |m~_k|^2 / 2);
  // e in four Kahan chains
  const float a2 = -0.5f * kLog2e * xnorm;
  float esum[4] = {0.f, 0.f, 0.f, 0.f}, ecmp[4] = {0.f, 0.f, 0.f, 0.f};
  const uint32_t id1 = idesc_tf32(kRows, kTK), id2 = idesc_tf32(kRows, kDP);
  uint32_t ph_a = 0, ph_b = 0, ph_g1 = 0, ph_g2 = 0;
  bool pend_a = false, pend_b = false, pend_g1 = false, pend_g2 = false;
  bool ok = true;
  auto load_a = [&](int t, bool first) {
    if (tid == 0) {
      const unsigned char *img = img_model + (size_t)t * kImgTile;
      mbar_expect_tx(bar_a, kMBytes + kMncBytes + (first ? kXBytes : 0));
      if (first) bulk_g2s(s_base + kOffX, img_atoms + (size_t)blockIdx.x * kXBytes, kXBytes, bar_a);
      bulk_g2s(s_base + kOffM, img, kMBytes, bar_a);
      bulk_g2s(s_base + kOffMnc + (t & 1) * kMncBytes, img + 2 * kMBytes, kMncBytes, bar_a);
    }
    pend_a = true;
  };
  auto load_b = [&](int t) {
    if (tid == 0) {
      mbar_expect_tx(bar_b, kMBytes);
      bulk_g2s(s_base + kOffMT, img_model + (size_t)t * kImgTile + kMBytes, kMBytes, bar_b);
    }
    pend_b = true;
  };
  if (ntiles > 0) {
    load_a(0, true);
    load_b(0);
  }
  for (int t = 0; t < ntiles && ok; ++t) {
    const float *smn = reinterpret_cast<const float *>(sm + kOffMnc + (t & 1) * kMncBytes);
    const float *sc = smn + kTK;
    ok = mbar_wait(bar_a, ph_a, flags);
    if (ok) {
      ph_a ^= 1;
      pend_a = false;
    }
    if (!__syncthreads_and(ok)) break;
    // GEMM1: C1[128 x 64] = x~ . m~ over K = 64 (8 steps of 8)
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int kk = 0; kk < kDP / 8; ++kk) {
        const uint64_t ad = smem_desc(s_base + kOffX + kk * 256, 128, (kDP / 4) * 128);
        const uint64_t bd = smem_desc(s_base + kOffM + kk * 256, 128, (kDP / 4) * 128);
        umma_tf32(tC1, ad, bd, id1, kk > 0 ? 1u : 0u);
      }
      umma_commit(bar_g1);
    }
    pend_g1 = true;
    ok = mbar_wait(bar_g1, ph_g1, flags);
    if (ok) {
      ph_g1 ^= 1;
      pend_g1 = false;
    }
    if (!__syncthreads_and(ok)) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (t + 1 < ntiles) load_a(t + 1, false);
    // epilogue: w = c exp(-s/2), e += w, W tile (TF32) for GEMM2
    unsigned char *wt = sm + kOffW;
    constexpr int kHalfBlocks = kTK / 64;  // 32-column blocks per column half
#pragma unroll 1
    for (int cc = kHalfBlocks * half; cc < kHalfBlocks * (half + 1); ++cc) {
      float v[32];
      tmem_ld32(tC1 + lane_base + cc * 32, v);
#pragma unroll
      for (int g = 0; g < 8; ++g) {
        uint32_t pk[4];
        const float4 b4 = *reinterpret_cast<const float4 *>(smn + cc * 32 + g * 4);
        const float4 c4 = *reinterpret_cast<const float4 *>(sc + cc * 32 + g * 4);
        const float bv[4] = {b4.x, b4.y, b4.z, b4.w}, cv[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float w = cv[u] * ex2_approx(fmaf(v[g * 4 + u], kLog2e, a2 + bv[u]));
          const float y = w - ecmp[u];  // Kahan
          const float tt = esum[u] + y;
          ecmp[u] = (tt - esum[u]) - y;
          esum[u] = tt;
          pk[u] = to_tf32(w);
        }
        *reinterpret_cast<uint4 *>(wt + kmajor32(row, cc * 32 + g * 4, kTK / 4)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    ok = mbar_wait(bar_b, ph_b, flags);
    if (ok) {
      ph_b ^= 1;
      pend_b = false;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    if (!__syncthreads_and(ok)) break;
    // GEMM2: C2[128 x 64] += W . m~^T over K = 64 (8 steps of 8)
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int kk = 0; kk < kTK / 8; ++kk) {
        const uint64_t ad = smem_desc(s_base + kOffW + kk * 256, 128, (kTK / 4) * 128);
        const uint64_t bd = smem_desc(s_base + kOffMT + kk * 256, 128, (kTK / 4) * 128);
        umma_tf32(tC2, ad, bd, id2, (t > 0 || kk > 0) ? 1u : 0u);
      }
      umma_commit(bar_g2);
    }
    pend_g2 = true;
    ok = mbar_wait(bar_g2, ph_g2, flags);
    if (ok) {
      ph_g2 ^= 1;
      pend_g2 = false;
    }
    ok = __syncthreads_and(ok);
    if (ok && t + 1 < ntiles) load_b(t + 1);
  }
  if (ok) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    double *ep = reinterpret_cast<double *>(sm + kOffEp);
    double emine = 0.0;
#pragma unroll
    for (int u = 0; u < 4; ++u) emine += (double)esum[u] - (double)ecmp[u];
    if (half == 1) ep[row] = emine;
    __syncthreads();
    if (half == 0) ep[row] = emine + ep[row];
    __syncthreads();
    const double etot = ep[row];
    float c2[32];
    tmem_ld32(tC2 + lane_base + half * 32, c2);
    if (i < N) {
      if (half == 0) e_out[i] = etot;
      const float ef = (float)etot;
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const int d = half * 32 + k;
        if (d < D) dedg[(size_t)i * D + d] = -invth[d] * (xs[(size_t)i * kDP + d] * ef - c2[k]);
      }
    }
  } else if (tid == 0) {
    if (pend_a) mbar_wait(bar_a, ph_a, flags);
    if (pend_b) mbar_wait(bar_b, ph_b, flags);
    if (pend_g1) mbar_wait(bar_g1, ph_g1, flags);
    if (pend_g2) mbar_wait(bar_g2, ph_g2, flags);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "n"(kTmemCols)
                 : "memory");
}

// x'' = G / theta - mu (FP32, row-padded to 64), the TF32 tiles of x~ and
// |x~|^2 (of the rounded vector)
__global__ void k_tf32_prep_atoms(int N, int D, const float *__restrict__ G,
                                  const float *__restrict__ invth, const float *__restrict__ mu,
                                  float *__restrict__ xs, float *__restrict__ xn,
                                  unsigned char *__restrict__ img) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int ntile_rows = ((N + kRows - 1) / kRows) * kRows;
  if (i >= ntile_rows) return;
  unsigned char *tile = img + (size_t)(i / kRows) * kXBytes;
  const int r = i % kRows;
  float nrm = 0.f;
  for (int k0 = 0; k0 < kDP; k0 += 4) {
    uint32_t pk[4];
    for (int u = 0; u < 4; ++u) {
      const int d = k0 + u;
      float x = 0.f;
      if (i < N && d < D) x = G[(size_t)i * D + d] * invth[d] - mu[d];
      if (i < N) xs[(size_t)i * kDP + d] = x;
      pk[u] = to_tf32(x);
      const float xr = __uint_as_float(pk[u]);
      nrm += xr * xr;
    }
    *reinterpret_cast<uint4 *>(tile + kmajor32(r, k0, kDP / 4)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
  }
  if (i < N) xn[i] = nrm;
}

// host FP32 -> TF32, round to nearest even
float tf32_round(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) != 0x7f800000u) {
    u += 0xfffu + ((u >> 13) & 1u);
    u &= ~0x1fffu;
  }
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

}  // namespace

// The model's TF32 image: per sparse tile m~ (K-major over D), m~^T (K-major
// over the tile's points), b2 = -log2e |m~|^2 / 2 and c, plus mu.
gapgb_status build_tf32_image(gapgb_model *m, bool refresh) {
  if (m->d_tf32 && !refresh) return GAPGB_OK;
  const HostModel &h = m->host;
  const int M = h.M, D = h.D;
  if (D > kDP) {
    set_last_error("tensor-core GPR supports D <= 64");
    return GAPGB_ERR_CAP_EXCEEDED;
  }
  const int nt = (M + kTK - 1) / kTK;
  std::vector<double> mu(kDP, 0.0);
  for (int k = 0; k < M; ++k)
    for (int d = 0; d < D; ++d) mu[d] += h.mm[(size_t)k * D + d] / h.theta[d] / M;
  std::vector<unsigned char> img((size_t)nt * kImgTile, 0);
  for (int t = 0; t < nt; ++t) {
    unsigned char *T = img.data() + (size_t)t * kImgTile;
    float *mn = reinterpret_cast<float *>(T + 2 * kMBytes);
    float *cf = mn + kTK;
    for (int kk = 0; kk < kTK; ++kk) {
      const int k = t * kTK + kk;
      if (k >= M) continue;
      double nrm = 0.0;
      for (int d = 0; d < kDP; ++d) {
        const double v = (d < D) ? h.mm[(size_t)k * D + d] / h.theta[d] - mu[d] : 0.0;
        const float vr = tf32_round((float)v);
        nrm += (double)vr * vr;
        std::memcpy(T + kmajor32(kk, d, kDP / 4), &vr, 4);            // GEMM1 B: rows = points
        std::memcpy(T + kMBytes + kmajor32(d, kk, kTK / 4), &vr, 4);  // GEMM2 B: rows = d
      }
      mn[kk] = (float)(-0.5 * 1.4426950408889634 * nrm);  // b2_k = -log2e |m~_k|^2 / 2
      cf[kk] = (float)h.coeff[k];
    }
  }
  std::vector<float> muf(kDP);
  for (int d = 0; d < kDP; ++d) muf[d] = (float)mu[d];
  const size_t bytes = img.size() + kDP * sizeof(float);
  if (!m->d_tf32) GAPGB_CUDA_TRY(cudaMalloc(&m->d_tf32, bytes));  // same size on a refresh
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_tf32, img.data(), img.size(), cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMemcpy((unsigned char *)m->d_tf32 + img.size(), muf.data(),
                            kDP * sizeof(float), cudaMemcpyHostToDevice));
  m->tf32_bytes = img.size();
  m->tf32_tiles = nt;
  return GAPGB_OK;
}

size_t tf32_atom_scratch_bytes(int N) {
  const size_t tiles = (size_t)(N + kRows - 1) / kRows;
  return tiles * kXBytes + (size_t)N * kDP * sizeof(float) + (size_t)N * sizeof(float) + 256;
}

void launch_gpr_tf32(gapgb_model *m, Workspace &ws, int N, cudaStream_t st, int a0, int a1) {
  const int D = m->host.D;
  if (a1 < 0) a1 = N;
  // the scratch layout is the whole batch's; the range's atoms start at tile a0 / 128
  const int tiles = (N + kRows - 1) / kRows;
  unsigned char *img_atoms = reinterpret_cast<unsigned char *>(ws.tc_scratch);
  float *xs = reinterpret_cast<float *>(img_atoms + (size_t)tiles * kXBytes);
  float *xn = xs + (size_t)N * kDP;
  const float *mu = reinterpret_cast<const float *>((const unsigned char *)m->d_tf32 + m->tf32_bytes);
  const int n = a1 - a0, t0 = a0 / kRows, ct = (n + kRows - 1) / kRows;
  if (n <= 0) return;
  unsigned char *img_r = img_atoms + (size_t)t0 * kXBytes;
  float *xs_r = xs + (size_t)a0 * kDP, *xn_r = xn + a0;
  k_tf32_prep_atoms<<<(ct * kRows + 127) / 128, 128, 0, st>>>(
      n, D, (const float *)ws.G + (size_t)a0 * D, m->d_invth32, mu, xs_r, xn_r, img_r);
  kernel_smem((const void *)k_gpr_tf32, kSmem, true);
  k_gpr_tf32<<<ct, kThreads, kSmem, st>>>(n, m->tf32_tiles, (const unsigned char *)m->d_tf32,
                                          img_r, xs_r, xn_r, m->d_invth32, D, ws.e + a0,
                                          (float *)ws.dedg + (size_t)a0 * D, ws.d_flags);
}

}  // namespace gapgb
