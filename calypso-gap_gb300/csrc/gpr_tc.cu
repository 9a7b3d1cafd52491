// gpr_tc.cu - the sparse-GPR contraction on the 5th-generation tensor cores.
//
// Same quantities as gpr.cu (GET_COV and the energy / dE/dG loops of
// FGAP_CALC, gappy/libgap/gap_calc.f90:143-166, 268-288), computed as two
// GEMMs with split-BF16 operands and FP32 accumulation in tensor memory:
//
//   centred, scaled descriptors  x'' = x/theta - mu,  m'' = m/theta - mu
//   (mu = mean of the sparse points; differences are unchanged by centring)
//   s_ik  = |x''_i|^2 + |m''_k|^2 - 2 x''_i . m''_k
//   GEMM1 (N x M, K = D):  x''.m'' ~ xh.mh + xh.ml + xl.mh  (3-term BF16 split,
//                          x'' = xh + xl, m'' = mh + ml, every product exact in FP32)
//                          as two MMAs per K step: xh.[mh; ml] (N = 128) into
//                          columns [0, 64) and [64, 128), and xl.mh (N = 64)
//                          into [0, 64); the epilogue adds the two halves
//   w_ik  = c_k exp(-s_ik / 2),  e_i = sum_k w_ik  (compensated FP32, Kahan)
//   GEMM2 (N x D, K = M):  (W M'')_id ~ wh.mh + wh.ml + wl.mh, the same way:
//                          wh.[mhT; mlT] (N = 128) and wl.mhT (N = 64)
//   dE/dG_id = -(1/theta_d) (x''_id e_i - (W M'')_id)
//
// One CTA (8 warps) owns 128 atoms.  For each tile of 64 sparse points: one
// 1-D bulk copy brings the pre-arranged operand tiles into shared memory,
// one thread issues GEMM1 (8 tcgen05.mma, M=128 K=16, N=128 and N=64) into a
// TMEM accumulator, the eight warps read it back with tcgen05.ld (thread =
// atom row), form w, accumulate e and write wh/wl into shared memory as
// GEMM2's A operand, and one thread issues GEMM2 (8 tcgen05.mma) accumulating
// over all sparse tiles in a second TMEM region.  Fewer, wider MMAs: an
// N = 128 MMA takes about 1.3 times as long as an N = 64 one on GB300, so the
// 16 MMAs of a tile take about 0.76 times as long as 24 N = 64 MMAs.  The
// [mh; ml] and [mhT; mlT] pairs are adjacent 64-row blocks in shared memory,
// which is the 128-row B operand of the same canonical layout.
//
// Operand tiles use the no-swizzle K-major canonical layout: 8-row x 16-byte
// core matrices, K-adjacent cores 128 B apart (LBO), 8-row groups
// (K/8)*128 B apart (SBO).  The model's tiles are built once on the host in
// that layout, so a tile is a contiguous block and needs no tensor map.
//
// Every mbarrier wait is bounded; a wait that gives up sets an error flag,
// the CTA skips the rest of its work, frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <cstring>

#include "gapgb_internal.h"
#include "tc_util.cuh"

namespace gapgb {
namespace {

using namespace tc;

constexpr int kRows = 128;   // atoms per CTA (UMMA M)
constexpr int kTileK = 64;   // sparse points per tile (GEMM1 N, GEMM2 K)
constexpr int kDP = 64;      // padded descriptor length (GEMM1 K, GEMM2 N)
constexpr int kXBytes16 = kRows * kDP * 2;           // 128 x 64 bf16: 16 KB
constexpr int kMBytes16 = kTileK * kDP * 2;          // 64 x 64 bf16: 8 KB
constexpr int kWBytes = kRows * kTileK * 2;          // 128 x 64 bf16: 16 KB
// per sparse tile image: mh, ml (64 x 64), mhT, mlT (64 x 64), b2[64], c[64]
constexpr int kImgTile = 4 * kMBytes16 + 2 * kTileK * 4;     // 32.5 KB
constexpr int kImgAtoms = 2 * kXBytes16;                      // xh, xl per 128 atoms

// shared memory map (bytes from the 1024-aligned base); about 99 KB, so two
// CTAs share an SM and one's GEMMs run under the other's epilogue
constexpr int kOffXh = 0;
constexpr int kOffXl = kOffXh + kXBytes16;
constexpr int kOffImg = kOffXl + kXBytes16;              // one sparse tile image
constexpr int kOffMh = kOffImg;
constexpr int kOffMl = kOffMh + kMBytes16;
constexpr int kOffMhT = kOffMl + kMBytes16;
constexpr int kOffMlT = kOffMhT + kMBytes16;
// [mh; ml] and [mhT; mlT] as one 128-row B operand: the second block starts
// eight 8-row groups (the canonical layout's SBO apart) after the first
static_assert(kOffMl - kOffMh == 8 * (kDP / 8) * 128, "mh / ml not one 128-row operand");
static_assert(kOffMlT - kOffMhT == 8 * (kTileK / 8) * 128, "mhT / mlT not one 128-row operand");
constexpr int kOffMnc = kOffMlT + kMBytes16;             // b2 and c, two tiles
constexpr int kMncBytes = 2 * kTileK * 4;                 // one tile's mn and c
constexpr int kOffWh = kOffMnc + 2 * kMncBytes;
constexpr int kOffWl = kOffWh + kWBytes;
constexpr int kOffBar = kOffWl + kWBytes;                 // 3 mbarriers + tmem base
constexpr int kOffEp = kOffBar + 64;                      // partial energies [128] (FP64)
constexpr int kSmemBytes = kOffEp + kRows * 8 + 1024;     // + alignment slack
constexpr int kGprThreads = 256;  // warps w and w + 4 share TMEM lanes and split the columns
constexpr int kTmemCols = 256;    // C1 and C2, two 64-column halves each

__global__ void __launch_bounds__(kGprThreads, 2)
    k_gpr_tc(int N, int ntiles, const unsigned char *__restrict__ img_model,
             const unsigned char *__restrict__ img_atoms, const float *__restrict__ xs,
             const float *__restrict__ xn, const float *__restrict__ invth, int D,
             double *__restrict__ e_out, float *__restrict__ dedg, int *__restrict__ flags) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>(
      ((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, half = warp >> 2;  // TMEM lane quadrant, column half
  const uint32_t s_base = smem_u32(sm);
  // bar_a: atoms (first tile), mh / ml and mn / c of a tile; bar_b: mhT / mlT
  const uint32_t bar_a = s_base + kOffBar, bar_g1 = bar_a + 8, bar_g2 = bar_a + 16,
                 bar_b = bar_a + 24;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + kOffBar + 32);
  int *abort_flag = reinterpret_cast<int *>(sm + kOffBar + 40);
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
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t tC1 = tmem, tC2 = tmem + 2 * kTileK;
  const uint32_t lane_base = (uint32_t)(quad * 32) << 16;  // this warp's TMEM lanes
  const int row = quad * 32 + lane;                         // atom row of this thread
  const int i = blockIdx.x * kRows + row;
  const float xnorm = (i < N) ? xn[i] : 0.f;
  // w = c exp(-s/2) = c 2^(log2e v + a2_i + b2_k) with a2_i = -log2e |x''_i|^2 / 2
  // and b2_k = -log2e |m''_k|^2 / 2 (the image stores b2): one add, one FMA
  // and ex2 per element.  e = sum w: each thread sums its 32 elements of a
  // tile into four plain partial sums (8 elements each), which enter four
  // independent Kahan chains once per tile.
  const float a2 = -0.5f * kLog2e * xnorm;
  float esum[4] = {0.f, 0.f, 0.f, 0.f}, ecmp[4] = {0.f, 0.f, 0.f, 0.f};
  // N = 128: [mh; ml] (GEMM1) or [mhT; mlT] (GEMM2); N = 64: mh or mhT alone
  const uint32_t id_pair = instr_desc(kRows, 128), id1 = instr_desc(kRows, kTileK),
                 id2 = instr_desc(kRows, kDP);
  uint32_t ph_a = 0, ph_b = 0, ph_g1 = 0, ph_g2 = 0;
  bool pend_a = false, pend_b = false, pend_g1 = false, pend_g2 = false;
  bool ok = true;
  // two-stage copy pipeline: a tile's GEMM1 operands (mh, ml, mn, c) load
  // while the previous tile's epilogue and GEMM2 run, its GEMM2 operands
  // (mhT, mlT) while its own GEMM1 and epilogue run
  auto load_a = [&](int t, bool first) {
    if (tid == 0) {
      const unsigned char *img = img_model + (size_t)t * kImgTile;
      mbar_expect_tx(bar_a, 2 * kMBytes16 + kMncBytes + (first ? kImgAtoms : 0));
      if (first)
        bulk_g2s(s_base + kOffXh, img_atoms + (size_t)blockIdx.x * kImgAtoms, kImgAtoms, bar_a);
      bulk_g2s(s_base + kOffMh, img, 2 * kMBytes16, bar_a);
      bulk_g2s(s_base + kOffMnc + (t & 1) * kMncBytes, img + 4 * kMBytes16, kMncBytes, bar_a);
    }
    pend_a = true;
  };
  auto load_b = [&](int t) {
    if (tid == 0) {
      mbar_expect_tx(bar_b, 2 * kMBytes16);
      bulk_g2s(s_base + kOffMhT, img_model + (size_t)t * kImgTile + 2 * kMBytes16,
               2 * kMBytes16, bar_b);
    }
    pend_b = true;
  };
  if (ntiles > 0) {
    load_a(0, true);
    load_b(0);
  }
  for (int t = 0; t < ntiles && ok; ++t) {
    const float *smn = reinterpret_cast<const float *>(sm + kOffMnc + (t & 1) * kMncBytes);
    const float *sc = smn + kTileK;
    ok = mbar_wait(bar_a, ph_a, flags);
    if (ok) {
      ph_a ^= 1;
      pend_a = false;
    }
    if (!__syncthreads_and(ok)) break;
    // GEMM1: C1[:, 0:64] + C1[:, 64:128] = xh.mh + xh.ml + xl.mh over K = 64
    // (4 steps of 16): xh.[mh; ml] into both halves, then xl.mh into the first
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a_off[2] = {kOffXh, kOffXl};
      for (int p = 0; p < 2; ++p)
        for (int kk = 0; kk < kDP / 16; ++kk) {
          const uint64_t ad = smem_desc(s_base + a_off[p] + kk * 256, 128, (kDP / 8) * 128);
          const uint64_t bd = smem_desc(s_base + kOffMh + kk * 256, 128, (kDP / 8) * 128);
          umma(tC1, ad, bd, p == 0 ? id_pair : id1, (p > 0 || kk > 0) ? 1u : 0u);
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
    // mh / ml are free again: the next tile's GEMM1 operands start loading
    if (t + 1 < ntiles) load_a(t + 1, false);
    // epilogue 1: w = c exp(-s/2), e += w, W tile (bf16 hi / lo) for GEMM2
    unsigned char *wh = sm + kOffWh, *wl = sm + kOffWl;
    constexpr int kHalfBlocks = kTileK / 64;  // 32-column blocks per column half
#pragma unroll 1
    for (int cc = kHalfBlocks * half; cc < kHalfBlocks * (half + 1); ++cc) {
      float v[32];
      tmem_ld32_sum2(tC1 + lane_base + cc * 32, kTileK, v);
      float part[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        uint32_t hpk[4], lpk[4];
        const int kg = cc * 32 + g * 8;
        const float4 b0 = *reinterpret_cast<const float4 *>(smn + kg);
        const float4 b1 = *reinterpret_cast<const float4 *>(smn + kg + 4);
        const float4 c0 = *reinterpret_cast<const float4 *>(sc + kg);
        const float4 c1 = *reinterpret_cast<const float4 *>(sc + kg + 4);
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
        const float cv[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          float w2[2];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const int q = h * 2 + u;
            const float w = cv[q] * ex2_approx(fmaf(v[g * 8 + q], kLog2e, a2 + bv[q]));
            part[h] += w;
            w2[u] = w;
          }
          const __nv_bfloat162 hi = __floats2bfloat162_rn(w2[0], w2[1]);
          const float2 hf = __bfloat1622float2(hi);
          hpk[h] = *reinterpret_cast<const uint32_t *>(&hi);
          lpk[h] = pack_bf16(w2[0] - hf.x, w2[1] - hf.y);
        }
        const int k0 = cc * 32 + g * 8;
        const int off = kmajor_off(row, k0, kTileK / 8);
        *reinterpret_cast<uint4 *>(wh + off) = make_uint4(hpk[0], hpk[1], hpk[2], hpk[3]);
        *reinterpret_cast<uint4 *>(wl + off) = make_uint4(lpk[0], lpk[1], lpk[2], lpk[3]);
      }
#pragma unroll
      for (int h = 0; h < 4; ++h) {  // Kahan
        const float y = part[h] - ecmp[h];
        const float tt = esum[h] + y;
        ecmp[h] = (tt - esum[h]) - y;
        esum[h] = tt;
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
    // GEMM2: C2[:, 0:64] + C2[:, 64:128] += wh.mhT + wh.mlT + wl.mhT over
    // K = 64 (4 steps of 16): wh.[mhT; mlT] into both halves, wl.mhT into the first
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a_off[2] = {kOffWh, kOffWl};
      for (int p = 0; p < 2; ++p)
        for (int kk = 0; kk < kTileK / 16; ++kk) {
          const uint64_t ad = smem_desc(s_base + a_off[p] + kk * 256, 128, (kTileK / 8) * 128);
          const uint64_t bd = smem_desc(s_base + kOffMhT + kk * 256, 128, (kTileK / 8) * 128);
          umma(tC2, ad, bd, p == 0 ? id_pair : id2, (t > 0 || p > 0 || kk > 0) ? 1u : 0u);
        }
      umma_commit(bar_g2);
    }
    pend_g2 = true;
    ok = mbar_wait(bar_g2, ph_g2, flags);  // operands are overwritten next tile
    if (ok) {
      ph_g2 ^= 1;
      pend_g2 = false;
    }
    ok = __syncthreads_and(ok);
    if (ok && t + 1 < ntiles) load_b(t + 1);
  }
  if (ok) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // the two column halves' partial energies, summed in a fixed order
    double *ep = reinterpret_cast<double *>(sm + kOffEp);
    double emine = 0.0;
#pragma unroll
    for (int h = 0; h < 4; ++h) emine += (double)esum[h] - (double)ecmp[h];
    if (half == 1) ep[row] = emine;
    __syncthreads();
    if (half == 0) ep[row] = emine + ep[row];
    __syncthreads();
    const double etot = ep[row];
    float c2[32];
    tmem_ld32_sum2(tC2 + lane_base + half * 32, kDP, c2);
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
    // a wait gave up: give the outstanding copy / MMA phases one more bounded
    // wait before the tensor memory and shared memory are released
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

// x'' = G / theta - mu (FP32, row-padded to 64), |x''|^2, and the xh/xl tiles
__global__ void k_tc_prep_atoms(int N, int D, const float *__restrict__ G,
                                const float *__restrict__ invth, const float *__restrict__ mu,
                                float *__restrict__ xs, float *__restrict__ xn,
                                unsigned char *__restrict__ img) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int ntile_rows = ((N + kRows - 1) / kRows) * kRows;
  if (i >= ntile_rows) return;
  unsigned char *tile = img + (size_t)(i / kRows) * kImgAtoms;
  const int r = i % kRows;
  float nrm = 0.f;
  for (int k0 = 0; k0 < kDP; k0 += 8) {
    uint32_t hp[4], lp[4];
    for (int h = 0; h < 4; ++h) {
      float x2[2];
      for (int u = 0; u < 2; ++u) {
        const int d = k0 + h * 2 + u;
        float x = 0.f;
        if (i < N && d < D) x = G[(size_t)i * D + d] * invth[d] - mu[d];
        if (i < N) xs[(size_t)i * kDP + d] = x;
        nrm += x * x;
        x2[u] = x;
      }
      const __nv_bfloat162 hi = __floats2bfloat162_rn(x2[0], x2[1]);
      const float2 hf = __bfloat1622float2(hi);
      hp[h] = *reinterpret_cast<const uint32_t *>(&hi);
      lp[h] = pack_bf16(x2[0] - hf.x, x2[1] - hf.y);
    }
    const int off = kmajor_off(r, k0, kDP / 8);
    *reinterpret_cast<uint4 *>(tile + off) = make_uint4(hp[0], hp[1], hp[2], hp[3]);
    *reinterpret_cast<uint4 *>(tile + kXBytes16 + off) = make_uint4(lp[0], lp[1], lp[2], lp[3]);
  }
  if (i < N) xn[i] = nrm;
}

// host-side bf16 (round to nearest even) for the model image
uint16_t bf16_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)(u >> 16);  // inf / nan
  const uint32_t lsb = (u >> 16) & 1u;
  u += 0x7fffu + lsb;
  return (uint16_t)(u >> 16);
}
float bf16_val(uint16_t b) {
  const uint32_t u = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

}  // namespace

size_t tc_smem_bytes() { return kSmemBytes; }

// Builds the model's tensor-core image: per sparse tile mh, ml (K-major over
// D), mhT, mlT (K-major over the tile's points), b2 = -log2e |m''|^2 / 2 and c
// (FP32), plus mu.
gapgb_status build_tc_image(gapgb_model *m, bool refresh) {
  if (m->d_tc && !refresh) return GAPGB_OK;
  const HostModel &h = m->host;
  const int M = h.M, D = h.D;
  if (D > kDP) {
    set_last_error("tensor-core GPR supports D <= 64");
    return GAPGB_ERR_CAP_EXCEEDED;
  }
  const int nt = (M + kTileK - 1) / kTileK;
  std::vector<double> mu(kDP, 0.0);
  std::vector<double> mm2((size_t)M * kDP, 0.0);
  for (int k = 0; k < M; ++k)
    for (int d = 0; d < D; ++d) {
      mm2[(size_t)k * kDP + d] = h.mm[(size_t)k * D + d] / h.theta[d];
      mu[d] += mm2[(size_t)k * kDP + d] / M;
    }
  std::vector<unsigned char> img((size_t)nt * kImgTile, 0);
  for (int t = 0; t < nt; ++t) {
    unsigned char *T = img.data() + (size_t)t * kImgTile;
    float *mn = reinterpret_cast<float *>(T + 4 * kMBytes16);
    float *cf = mn + kTileK;
    for (int kk = 0; kk < kTileK; ++kk) {
      const int k = t * kTileK + kk;
      if (k >= M) continue;
      double nrm = 0.0;
      for (int d = 0; d < kDP; ++d) {
        const double v = (d < D) ? mm2[(size_t)k * kDP + d] - mu[d] : 0.0;
        nrm += v * v;
        const uint16_t hb = bf16_bits((float)v);
        const uint16_t lb = bf16_bits((float)(v - (double)bf16_val(hb)));
        // GEMM1 B operand: rows = sparse points, K = descriptor components
        std::memcpy(T + kmajor_off(kk, d, kDP / 8), &hb, 2);
        std::memcpy(T + kMBytes16 + kmajor_off(kk, d, kDP / 8), &lb, 2);
        // GEMM2 B operand: rows = descriptor components, K = sparse points
        std::memcpy(T + 2 * kMBytes16 + kmajor_off(d, kk, kTileK / 8), &hb, 2);
        std::memcpy(T + 3 * kMBytes16 + kmajor_off(d, kk, kTileK / 8), &lb, 2);
      }
      mn[kk] = (float)(-0.5 * 1.4426950408889634 * nrm);  // b2_k = -log2e |m''_k|^2 / 2
      cf[kk] = (float)h.coeff[k];
    }
  }
  std::vector<float> muf(kDP);
  for (int d = 0; d < kDP; ++d) muf[d] = (float)mu[d];
  const size_t bytes = img.size() + kDP * sizeof(float);
  if (!m->d_tc) GAPGB_CUDA_TRY(cudaMalloc(&m->d_tc, bytes));  // same size on a refresh
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_tc, img.data(), img.size(), cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMemcpy((unsigned char *)m->d_tc + img.size(), muf.data(), kDP * sizeof(float),
                            cudaMemcpyHostToDevice));
  m->tc_bytes = img.size();
  m->tc_tiles = nt;
  return GAPGB_OK;
}

size_t tc_atom_scratch_bytes(int N) {
  const size_t tiles = (size_t)(N + kRows - 1) / kRows;
  return tiles * kImgAtoms + (size_t)N * kDP * sizeof(float) + (size_t)N * sizeof(float) + 1024;
}

void launch_gpr_tc(gapgb_model *m, Workspace &ws, int N, cudaStream_t st, int a0, int a1) {
  const int D = m->host.D;
  if (a1 < 0) a1 = N;
  // the scratch layout is the whole batch's; the range's atoms start at tile a0 / 128
  const int tiles = (N + kRows - 1) / kRows;
  unsigned char *img_atoms = reinterpret_cast<unsigned char *>(ws.tc_scratch);
  float *xs = reinterpret_cast<float *>(img_atoms + (size_t)tiles * kImgAtoms);
  float *xn = xs + (size_t)N * kDP;
  const float *mu = reinterpret_cast<const float *>((const unsigned char *)m->d_tc + m->tc_bytes);
  const int n = a1 - a0, t0 = a0 / kRows, ct = (n + kRows - 1) / kRows;
  if (n <= 0) return;
  unsigned char *img_r = img_atoms + (size_t)t0 * kImgAtoms;
  float *xs_r = xs + (size_t)a0 * kDP, *xn_r = xn + a0;
  k_tc_prep_atoms<<<(ct * kRows + 127) / 128, 128, 0, st>>>(
      n, D, (const float *)ws.G + (size_t)a0 * D, m->d_invth32, mu, xs_r, xn_r, img_r);
  kernel_smem((const void *)k_gpr_tc, kSmemBytes, true);
  k_gpr_tc<<<ct, kGprThreads, kSmemBytes, st>>>(n, m->tc_tiles, (const unsigned char *)m->d_tc,
                                                img_r, xs_r, xn_r, m->d_invth32, D, ws.e + a0,
                                                (float *)ws.dedg + (size_t)a0 * D, ws.d_flags);
}

}  // namespace gapgb
