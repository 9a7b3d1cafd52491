// mlp_tc.cu - the surrogate's committee forward + input gradient on the
// 5th-generation tensor cores (inference only; training uses mlp.cu's
// kernels).  For H = 128 hidden units and D <= 64 descriptor components.
//
// One CTA (4 warps, thread = atom row) runs one committee member over a
// stream of 128-row tiles of the species-sorted rows; tiles are sorted by
// species, so a CTA reloads its member's weight image (96 KB: W1, W2, W2^T,
// W1^T as BF16 K-major canonical tiles) at most once per species.  Per tile,
// with accumulators in tensor memory (512 columns: Z1 | Z2, then U | G):
//   GEMM1  Z1 = X W1^T          (M 128, N 128, K 64)
//   epi 1  a1 = silu(z1 + b1)   -> BF16 A tile
//   GEMM2  Z2 = a1 W2^T         (M 128, N 128, K 128)
//   epi 2  y = w3 . silu(z2 + b2) + b3;  d2 = w3 o silu'(z2 + b2) -> BF16
//   GEMM3  U = d2 W2            (B = W2^T image, M 128, N 128, K 128)
//   epi 3  d1 = silu'(z1 + b1) o U -> BF16
//   GEMM4  G = d1 W1            (B = W1^T image, M 128, N 64, K 128)
//   epi 4  y and dy/dx rows to global memory (member-major, as mlp.cu)
// Eight warps: warps w and w + 4 read the same TMEM lanes (rows) and split
// the columns; b1, b2, w3, b3 travel in the weight image; the next tile's X
// is prefetched into a second buffer while the current tile is processed.
// The operands d2 and d1 are BF16 here (FP32 in the SIMT forward of
// mlp.cu): 2^-9 relative rounding of each element, far below the network's
// own error.  One thread issues the MMAs; every mbarrier wait is bounded
// and a wait that gives up raises the timeout flag, stops the CTA's work,
// frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "gapgb_internal.h"
#include "tc_util.cuh"

namespace gapgb {
namespace {

using namespace tc;

constexpr int kR = 128;   // rows per tile (UMMA M)
constexpr int kDp = 64;   // padded descriptor length
constexpr int kHid = 128; // hidden units
constexpr int kThreads = 256;  // 8 warps: warps w and w + 4 share TMEM lanes, split columns
constexpr int kXBytes = kR * kDp * 2;        // 16 KB
constexpr int kW1Bytes = kHid * kDp * 2;     // 16 KB
constexpr int kW2Bytes = kHid * kHid * 2;    // 32 KB
constexpr int kVecBytes = (3 * kHid + 4) * 4;                   // b1, b2, w3, b3 (FP32)
constexpr int kWImg = 2 * kW1Bytes + 2 * kW2Bytes + kVecBytes;  // one (member, species) image
constexpr int kOffVec = 2 * kW1Bytes + 2 * kW2Bytes;            // within the image
// shared memory map (from the 1024-aligned base)
constexpr int kOffX0 = 0;                    // X tiles, double-buffered
constexpr int kOffX1 = kOffX0 + kXBytes;
constexpr int kOffW1 = kOffX1 + kXBytes;     // weight image: W1, W2, W2T, W1T, vectors
constexpr int kOffW2 = kOffW1 + kW1Bytes;
constexpr int kOffW2T = kOffW2 + kW2Bytes;
constexpr int kOffW1T = kOffW2T + kW2Bytes;
constexpr int kOffA = (kOffW1 + kWImg + 1023) / 1024 * 1024;  // a1, then d1 (128 x 128)
constexpr int kOffDd = kOffA + kW2Bytes;                       // d2 (128 x 128)
constexpr int kPitch = kDp + 1;                                // dy/dx staging pitch (floats)
static_assert(kR * kPitch * 4 <= 2 * kW2Bytes, "dy/dx staging fits the A and Dd tiles");
constexpr int kOffY = kOffDd + kW2Bytes;                       // partial y [2][128]
constexpr int kOffBar = kOffY + 2 * kR * 4;
constexpr int kMlpSmem = kOffBar + 64 + 1024;
static_assert(kWImg % 16 == 0, "bulk copies move multiples of 16 bytes");

// logistic function with the fast reciprocal (2-ulp division; the results
// become BF16 operands or FP32 sums)
__device__ __forceinline__ float sig(float z) { return __fdividef(1.f, 1.f + __expf(-z)); }

// weight image of every (member, species) block: W1 [h][d], W2 [i][j],
// W2^T [j][i], W1^T [d][h] as K-major canonical BF16 tiles (rows = UMMA N),
// then b1, b2, w3, b3 in FP32
__global__ void k_mlp_w_image(int nblk, int D, size_t P, size_t offW1, size_t offW2, size_t offb1,
                              size_t offb2, size_t offw3, size_t offb3,
                              const __nv_bfloat16 *__restrict__ w16, const float *__restrict__ w32,
                              unsigned char *__restrict__ img) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t per = (size_t)kHid * kDp + (size_t)kHid * kHid + kHid;  // W1, W2 elements, vectors
  if (t >= per * nblk) return;
  const int b = (int)(t / per);
  const size_t e = t - (size_t)b * per;
  const __nv_bfloat16 *w = w16 + (size_t)b * P;
  const float *wf = w32 + (size_t)b * P;
  unsigned char *o = img + (size_t)b * kWImg;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  if (e < (size_t)kHid * kDp) {
    const int h = (int)(e / kDp), d = (int)(e % kDp);
    const __nv_bfloat16 v = d < D ? w[offW1 + (size_t)h * D + d] : zero;
    *reinterpret_cast<__nv_bfloat16 *>(o + kmajor_off(h, d, kDp / 8)) = v;  // W1 (N = h, K = d)
    *reinterpret_cast<__nv_bfloat16 *>(o + kW1Bytes + 2 * kW2Bytes + kmajor_off(d, h, kHid / 8)) =
        v;  // W1^T (N = d, K = h)
  } else if (e < (size_t)kHid * kDp + (size_t)kHid * kHid) {
    const size_t f = e - (size_t)kHid * kDp;
    const int i = (int)(f / kHid), j = (int)(f % kHid);
    const __nv_bfloat16 v = w[offW2 + (size_t)i * kHid + j];
    *reinterpret_cast<__nv_bfloat16 *>(o + kW1Bytes + kmajor_off(i, j, kHid / 8)) = v;  // W2
    *reinterpret_cast<__nv_bfloat16 *>(o + kW1Bytes + kW2Bytes + kmajor_off(j, i, kHid / 8)) =
        v;  // W2^T (N = j, K = i)
  } else {
    const int h = (int)(e - (size_t)kHid * kDp - (size_t)kHid * kHid);
    float *vec = reinterpret_cast<float *>(o + kOffVec);
    vec[h] = wf[offb1 + h];
    vec[kHid + h] = wf[offb2 + h];
    vec[2 * kHid + h] = wf[offw3 + h];
    if (h < 4) vec[3 * kHid + h] = h == 0 ? wf[offb3] : 0.f;
  }
}

// standardised BF16 rows of the species-sorted order in the K-major X tiles
// (idx < 0: padding row, zeros); one thread per (row, 8 components)
__global__ void k_mlp_x_image(int Mpad, int D, const int *__restrict__ idx,
                              const float *__restrict__ G, const float *__restrict__ mu,
                              const float *__restrict__ isig, unsigned char *__restrict__ img) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= Mpad * (kDp / 8)) return;
  const int row = t / (kDp / 8), d0 = (t % (kDp / 8)) * 8;
  const int a = idx[row];
  uint32_t pk[4];
#pragma unroll
  for (int h = 0; h < 4; ++h) {
    float v[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int d = d0 + 2 * h + u;
      v[u] = (a >= 0 && d < D) ? (G[(size_t)a * D + d] - mu[d]) * isig[d] : 0.f;
    }
    pk[h] = pack_bf16(v[0], v[1]);
  }
  unsigned char *tile = img + (size_t)(row / kR) * kXBytes;
  *reinterpret_cast<uint4 *>(tile + kmajor_off(row % kR, d0, kDp / 8)) =
      make_uint4(pk[0], pk[1], pk[2], pk[3]);
}

struct MlpTcArgs {
  int ntiles, Mpad, D, nsp;
  const unsigned char *wimg;     // weight images [members * nsp]
  const unsigned char *ximg;     // X tiles [ntiles]
  const int *tile_sp64;          // species of each 64-row tile (-1: beyond the rows)
  float *y, *gx;                 // [members][Mpad], [members][Mpad][D]
  int *flags;
};

__global__ void __launch_bounds__(kThreads, 1) k_mlp_tc(MlpTcArgs a) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sm =
      reinterpret_cast<unsigned char *>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quad = warp & 3, half = warp >> 2;  // TMEM lane quadrant, column half
  const int r = quad * 32 + lane;                // row of the tile
  const int q = blockIdx.y;
  const uint32_t s_base = smem_u32(sm);
  const uint32_t bar_x0 = s_base + kOffBar, bar_x1 = bar_x0 + 8, bar_w = bar_x0 + 16,
                 bar_mma = bar_x0 + 24;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + kOffBar + 32);
  float *ypart = reinterpret_cast<float *>(sm + kOffY);
  const float *vb1 = reinterpret_cast<const float *>(sm + kOffW1 + kOffVec);
  const float *vb2 = vb1 + kHid, *vw3 = vb1 + 2 * kHid, *vb3 = vb1 + 3 * kHid;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(bar_x0, 1);
    mbar_init(bar_x1, 1);
    mbar_init(bar_w, 1);
    mbar_init(bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t tZ1 = tmem, tZ2 = tmem + 128, tG = tmem + 256;
  const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
  const uint32_t id128 = instr_desc(kR, 128), id64 = instr_desc(kR, 64);
  uint32_t ph_x0 = 0, ph_x1 = 0, ph_w = 0, ph_mma = 0;
  bool ok = true;
  int loaded = -1, buf = 0;
  bool pend0 = false, pend1 = false;  // X copies in flight, per buffer
  bool pending_w = false, pending_mma = false;
  auto valid_tile = [&](int t) { return t < a.ntiles && a.tile_sp64[2 * t] >= 0; };
  auto load_x = [&](int t, int b) {
    if (tid == 0) {
      const uint32_t bar = b ? bar_x1 : bar_x0;
      mbar_expect_tx(bar, kXBytes);
      bulk_g2s(s_base + (b ? kOffX1 : kOffX0), a.ximg + (size_t)t * kXBytes, kXBytes, bar);
    }
    if (b) pend1 = true; else pend0 = true;
  };
  // MMA issue (one thread) and the bounded wait on its completion
  auto gemm = [&](uint32_t dt, int offA, int offB, int kcores, int ksteps, uint32_t idesc) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int kk = 0; kk < ksteps; ++kk) {
        const uint64_t ad = smem_desc(s_base + offA + kk * 256, 128, kcores * 128);
        const uint64_t bd = smem_desc(s_base + offB + kk * 256, 128, kcores * 128);
        umma(dt, ad, bd, idesc, kk > 0 ? 1u : 0u);
      }
      umma_commit(bar_mma);
    }
    pending_mma = true;
    ok = mbar_wait(bar_mma, ph_mma, a.flags);
    if (ok) {
      ph_mma ^= 1;
      pending_mma = false;
    }
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  };
  if (valid_tile(blockIdx.x)) load_x(blockIdx.x, 0);
  for (int t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x) {
    const int sp = a.tile_sp64[2 * t];
    if (sp < 0) break;  // padding tiles come last
    if (sp != loaded) {
      // every MMA reading the previous weights has completed (waited below)
      if (tid == 0) {
        mbar_expect_tx(bar_w, kWImg);
        bulk_g2s(s_base + kOffW1, a.wimg + (size_t)(q * a.nsp + sp) * kWImg, kWImg, bar_w);
      }
      loaded = sp;
      pending_w = true;
      ok = mbar_wait(bar_w, ph_w, a.flags);
      if (ok) {
        ph_w ^= 1;
        pending_w = false;
      }
      if (!__syncthreads_and(ok)) break;
    }
    ok = mbar_wait(buf ? bar_x1 : bar_x0, buf ? ph_x1 : ph_x0, a.flags);
    if (ok) {
      if (buf) { ph_x1 ^= 1; pend1 = false; } else { ph_x0 ^= 1; pend0 = false; }
    }
    if (!__syncthreads_and(ok)) break;
    const int row = t * kR + r;
    // GEMM1; its X buffer is then free, so the next tile's X is prefetched
    gemm(tZ1, buf ? kOffX1 : kOffX0, kOffW1, kDp / 8, kDp / 16, id128);
    if (!ok) break;
    if (valid_tile(t + gridDim.x)) load_x(t + gridDim.x, buf ^ 1);
    // epilogue 1: a1 = silu(z1 + b1), this thread's 64 columns
#pragma unroll 1
    for (int cc = 2 * half; cc < 2 * half + 2; ++cc) {
      float v[32];
      tmem_ld32(tZ1 + lane_base + cc * 32, v);
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        uint32_t pk[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int c0 = cc * 32 + g * 8 + 2 * h;
          const float z0 = v[g * 8 + 2 * h] + vb1[c0], z1 = v[g * 8 + 2 * h + 1] + vb1[c0 + 1];
          pk[h] = pack_bf16(z0 * sig(z0), z1 * sig(z1));
        }
        *reinterpret_cast<uint4 *>(sm + kOffA + kmajor_off(r, cc * 32 + g * 8, kHid / 8)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    // GEMM2 and epilogue 2: partial y, d2
    gemm(tZ2, kOffA, kOffW2, kHid / 8, kHid / 16, id128);
    if (!ok) break;
    float ysum = 0.f;
#pragma unroll 1
    for (int cc = 2 * half; cc < 2 * half + 2; ++cc) {
      float v[32];
      tmem_ld32(tZ2 + lane_base + cc * 32, v);
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        uint32_t pk[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          float d2v[2];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const int c = cc * 32 + g * 8 + 2 * h + u;
            const float z = v[g * 8 + 2 * h + u] + vb2[c];
            const float s = sig(z);
            ysum = fmaf(z * s, vw3[c], ysum);
            d2v[u] = vw3[c] * s * (1.f + z * (1.f - s));
          }
          pk[h] = pack_bf16(d2v[0], d2v[1]);
        }
        *reinterpret_cast<uint4 *>(sm + kOffDd + kmajor_off(r, cc * 32 + g * 8, kHid / 8)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    ypart[half * kR + r] = ysum;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    // GEMM3 (into the Z2 columns); the partial y are complete after its sync
    gemm(tZ2, kOffDd, kOffW2T, kHid / 8, kHid / 16, id128);
    if (!ok) break;
    if (half == 0 && row < a.Mpad) a.y[(size_t)q * a.Mpad + row] = ypart[r] + ypart[kR + r] + vb3[0];
    // epilogue 3: d1 = silu'(z1 + b1) o U
#pragma unroll 1
    for (int cc = 2 * half; cc < 2 * half + 2; ++cc) {
      float u[32], z[32];
      tmem_ld32(tZ2 + lane_base + cc * 32, u);
      tmem_ld32(tZ1 + lane_base + cc * 32, z);
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        uint32_t pk[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          float dv[2];
#pragma unroll
          for (int w = 0; w < 2; ++w) {
            const int k = g * 8 + 2 * h + w;
            const float zz = z[k] + vb1[cc * 32 + k];
            const float s = sig(zz);
            dv[w] = s * (1.f + zz * (1.f - s)) * u[k];
          }
          pk[h] = pack_bf16(dv[0], dv[1]);
        }
        *reinterpret_cast<uint4 *>(sm + kOffA + kmajor_off(r, cc * 32 + g * 8, kHid / 8)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    // GEMM4 and epilogue 4: dy/dx, this thread's 32 components
    gemm(tG, kOffA, kOffW1T, kHid / 8, kHid / 16, id64);
    if (!ok) break;
    // the tile's dy/dx rows go through shared memory (the A and Dd tiles are
    // free after GEMM4) with a row pitch of 65 floats, so the row-per-lane
    // writes and the coalesced read-out are both free of bank conflicts
    float gv[32];
    tmem_ld32(tG + lane_base + half * 32, gv);
    float *stage = reinterpret_cast<float *>(sm + kOffA);  // [128][kPitch]
#pragma unroll
    for (int d = 0; d < 32; ++d) stage[r * kPitch + half * 32 + d] = gv[d];
    __syncthreads();
    {
      const size_t base = ((size_t)q * a.Mpad + (size_t)t * kR) * a.D;
      const int n = kR * a.D;  // floats of the tile (rows t*128 .. t*128 + 127)
      for (int k = tid; k < n; k += kThreads) {
        const int rr = k / a.D, d = k - rr * a.D;
        a.gx[base + k] = stage[rr * kPitch + d];
      }
    }
    buf ^= 1;
  }
  if (!ok && tid == 0) {
    // a wait gave up: one more bounded wait for every phase that may still be
    // outstanding before the tensor and shared memory are released
    if (pend0) mbar_wait(bar_x0, ph_x0, a.flags);
    if (pend1) mbar_wait(bar_x1, ph_x1, a.flags);
    if (pending_w) mbar_wait(bar_w, ph_w, a.flags);
    if (pending_mma) mbar_wait(bar_mma, ph_mma, a.flags);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

}  // namespace

size_t mlp_tc_w_image_bytes(int nblk) { return (size_t)nblk * kWImg; }
size_t mlp_tc_x_image_bytes(int Mpad) { return (size_t)((Mpad + kR - 1) / kR) * kXBytes; }
bool mlp_tc_eligible(int D, int H) { return D <= kDp && H == kHid; }

void launch_mlp_w_image(int nblk, int D, size_t P, size_t offW1, size_t offW2, size_t offb1,
                        size_t offb2, size_t offw3, size_t offb3, const __nv_bfloat16 *w16,
                        const float *w32, unsigned char *img, cudaStream_t st) {
  const size_t n = ((size_t)kHid * kDp + (size_t)kHid * kHid + kHid) * nblk;
  k_mlp_w_image<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nblk, D, P, offW1, offW2, offb1,
                                                             offb2, offw3, offb3, w16, w32, img);
}

void launch_mlp_tc(int members, int nsp, int D, int Mpad, const unsigned char *wimg,
                   unsigned char *ximg, const int *idx, const float *G, const float *mu,
                   const float *isig, const int *tile_sp64, float *y, float *gx, int *flags,
                   cudaStream_t st) {
  const int nx = Mpad * (kDp / 8);
  k_mlp_x_image<<<(nx + 255) / 256, 256, 0, st>>>(Mpad, D, idx, G, mu, isig, ximg);
  const int sms = device_sms();
  const int ntiles = Mpad / kR;
  const int per_member = std::max(1, std::min(ntiles, (sms + members - 1) / members));
  MlpTcArgs a{ntiles, Mpad, D, nsp, wimg, ximg, tile_sp64, y, gx, flags};
  kernel_smem((const void *)k_mlp_tc, kMlpSmem);
  k_mlp_tc<<<dim3(per_member, members), kThreads, kMlpSmem, st>>>(a);
}

}  // namespace gapgb
