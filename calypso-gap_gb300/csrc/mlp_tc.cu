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
constexpr int kXBytes = kR * kDp * 2;        // 16 KB
constexpr int kW1Bytes = kHid * kDp * 2;     // 16 KB
constexpr int kW2Bytes = kHid * kHid * 2;    // 32 KB
constexpr int kWImg = 2 * kW1Bytes + 2 * kW2Bytes;  // W1, W2, W2T, W1T: 96 KB
// shared memory map (from the 1024-aligned base)
constexpr int kOffX = 0;
constexpr int kOffW1 = kOffX + kXBytes;
constexpr int kOffW2 = kOffW1 + kW1Bytes;
constexpr int kOffW2T = kOffW2 + kW2Bytes;
constexpr int kOffW1T = kOffW2T + kW2Bytes;
constexpr int kOffA = kOffW1T + kW1Bytes;     // a1, then d1 (128 x 128)
constexpr int kOffDd = kOffA + kW2Bytes;      // d2 (128 x 128)
constexpr int kOffBar = kOffDd + kW2Bytes;
constexpr int kMlpSmem = kOffBar + 64 + 1024;

__device__ __forceinline__ float sig(float z) { return 1.f / (1.f + __expf(-z)); }

// weight image of every (member, species) block: W1 [h][d], W2 [i][j],
// W2^T [j][i], W1^T [d][h], each a K-major canonical tile (rows = UMMA N)
__global__ void k_mlp_w_image(int nblk, int D, size_t P, size_t offW1, size_t offW2,
                              const __nv_bfloat16 *__restrict__ w16, unsigned char *__restrict__ img) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t per = (size_t)kHid * kDp + (size_t)kHid * kHid;  // elements of W1 and W2
  if (t >= per * nblk) return;
  const int b = (int)(t / per);
  const size_t e = t - (size_t)b * per;
  const __nv_bfloat16 *w = w16 + (size_t)b * P;
  unsigned char *o = img + (size_t)b * kWImg;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  if (e < (size_t)kHid * kDp) {
    const int h = (int)(e / kDp), d = (int)(e % kDp);
    const __nv_bfloat16 v = d < D ? w[offW1 + (size_t)h * D + d] : zero;
    *reinterpret_cast<__nv_bfloat16 *>(o + kmajor_off(h, d, kDp / 8)) = v;  // W1 (N = h, K = d)
    *reinterpret_cast<__nv_bfloat16 *>(o + kW1Bytes + 2 * kW2Bytes + kmajor_off(d, h, kHid / 8)) =
        v;  // W1^T (N = d, K = h)
  } else {
    const size_t f = e - (size_t)kHid * kDp;
    const int i = (int)(f / kHid), j = (int)(f % kHid);
    const __nv_bfloat16 v = w[offW2 + (size_t)i * kHid + j];
    *reinterpret_cast<__nv_bfloat16 *>(o + kW1Bytes + kmajor_off(i, j, kHid / 8)) = v;  // W2
    *reinterpret_cast<__nv_bfloat16 *>(o + kW1Bytes + kW2Bytes + kmajor_off(j, i, kHid / 8)) =
        v;  // W2^T (N = j, K = i)
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
  size_t P, offb1, offb2, offw3, offb3;
  const float *w;                // FP32 parameters (biases, w3, b3)
  const unsigned char *wimg;     // weight images [members * nsp]
  const unsigned char *ximg;     // X tiles [ntiles]
  const int *tile_sp64;          // species of each 64-row tile (-1: beyond the rows)
  float *y, *gx;                 // [members][Mpad], [members][Mpad][D]
  int *flags;
};

__global__ void __launch_bounds__(128, 1) k_mlp_tc(MlpTcArgs a) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sm =
      reinterpret_cast<unsigned char *>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int q = blockIdx.y;
  const uint32_t s_base = smem_u32(sm);
  const uint32_t bar_load = s_base + kOffBar, bar_mma = bar_load + 8;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + kOffBar + 32);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(bar_load, 1);
    mbar_init(bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t tZ1 = tmem, tZ2 = tmem + 128, tG = tmem + 256;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const uint32_t id128 = instr_desc(kR, 128), id64 = instr_desc(kR, 64);
  uint32_t ph_load = 0, ph_mma = 0;
  bool ok = true;
  int loaded = -1;
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
    ok = mbar_wait(bar_mma, ph_mma, a.flags);
    ph_mma ^= 1;
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  };
  for (int t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x) {
    const int sp = a.tile_sp64[2 * t];
    if (sp < 0) break;  // padding tiles come last
    const bool reload = sp != loaded;
    if (tid == 0) {
      mbar_expect_tx(bar_load, kXBytes + (reload ? kWImg : 0));
      bulk_g2s(s_base + kOffX, a.ximg + (size_t)t * kXBytes, kXBytes, bar_load);
      if (reload)
        bulk_g2s(s_base + kOffW1, a.wimg + (size_t)(q * a.nsp + sp) * kWImg, kWImg, bar_load);
    }
    loaded = sp;
    ok = mbar_wait(bar_load, ph_load, a.flags);
    ph_load ^= 1;
    if (!__syncthreads_and(ok)) break;
    const float *blk = a.w + (size_t)(q * a.nsp + sp) * a.P;
    const float *b1 = blk + a.offb1, *b2 = blk + a.offb2, *w3 = blk + a.offw3;
    const int row = t * kR + tid;
    // GEMM1 and epilogue 1: a1 = silu(z1 + b1)
    gemm(tZ1, kOffX, kOffW1, kDp / 8, kDp / 16, id128);
    if (!ok) break;
#pragma unroll 1
    for (int cc = 0; cc < 4; ++cc) {
      float v[32];
      tmem_ld32(tZ1 + lane_base + cc * 32, v);
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        uint32_t pk[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int c0 = cc * 32 + g * 8 + 2 * h;
          const float z0 = v[g * 8 + 2 * h] + b1[c0], z1 = v[g * 8 + 2 * h + 1] + b1[c0 + 1];
          pk[h] = pack_bf16(z0 * sig(z0), z1 * sig(z1));
        }
        *reinterpret_cast<uint4 *>(sm + kOffA + kmajor_off(tid, cc * 32 + g * 8, kHid / 8)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    // GEMM2 and epilogue 2: y, d2
    gemm(tZ2, kOffA, kOffW2, kHid / 8, kHid / 16, id128);
    if (!ok) break;
    float ysum = 0.f;
#pragma unroll 1
    for (int cc = 0; cc < 4; ++cc) {
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
            const float z = v[g * 8 + 2 * h + u] + b2[c];
            const float s = sig(z);
            ysum = fmaf(z * s, w3[c], ysum);
            d2v[u] = w3[c] * s * (1.f + z * (1.f - s));
          }
          pk[h] = pack_bf16(d2v[0], d2v[1]);
        }
        *reinterpret_cast<uint4 *>(sm + kOffDd + kmajor_off(tid, cc * 32 + g * 8, kHid / 8)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    if (row < a.Mpad) a.y[(size_t)q * a.Mpad + row] = ysum + blk[a.offb3];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    // GEMM3 (into the Z2 columns) and epilogue 3: d1 = silu'(z1 + b1) o U
    gemm(tZ2, kOffDd, kOffW2T, kHid / 8, kHid / 16, id128);
    if (!ok) break;
#pragma unroll 1
    for (int cc = 0; cc < 4; ++cc) {
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
            const float zz = z[k] + b1[cc * 32 + k];
            const float s = sig(zz);
            dv[w] = s * (1.f + zz * (1.f - s)) * u[k];
          }
          pk[h] = pack_bf16(dv[0], dv[1]);
        }
        *reinterpret_cast<uint4 *>(sm + kOffA + kmajor_off(tid, cc * 32 + g * 8, kHid / 8)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    // GEMM4 and epilogue 4: dy/dx rows
    gemm(tG, kOffA, kOffW1T, kHid / 8, kHid / 16, id64);
    if (!ok) break;
    float gv[64];
    tmem_ld32(tG + lane_base, gv);
    tmem_ld32(tG + lane_base + 32, gv + 32);
    if (row < a.Mpad) {
      float *o = a.gx + ((size_t)q * a.Mpad + row) * a.D;
#pragma unroll
      for (int d = 0; d < kDp; ++d)
        if (d < a.D) o[d] = gv[d];
    }
  }
  if (!ok && tid == 0) {
    // a wait gave up: one more bounded wait for the outstanding phases
    // before the tensor memory and shared memory are released
    mbar_wait(bar_load, ph_load, a.flags);
    mbar_wait(bar_mma, ph_mma, a.flags);
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

void launch_mlp_w_image(int nblk, int D, size_t P, size_t offW1, size_t offW2,
                        const __nv_bfloat16 *w16, unsigned char *img, cudaStream_t st) {
  const size_t n = ((size_t)kHid * kDp + (size_t)kHid * kHid) * nblk;
  k_mlp_w_image<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nblk, D, P, offW1, offW2, w16, img);
}

void launch_mlp_tc(int members, int nsp, int D, int Mpad, size_t P, size_t offb1, size_t offb2,
                   size_t offw3, size_t offb3, const float *w, const unsigned char *wimg,
                   unsigned char *ximg, const int *idx, const float *G, const float *mu,
                   const float *isig, const int *tile_sp64, float *y, float *gx, int *flags,
                   cudaStream_t st) {
  const int nx = Mpad * (kDp / 8);
  k_mlp_x_image<<<(nx + 255) / 256, 256, 0, st>>>(Mpad, D, idx, G, mu, isig, ximg);
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int ntiles = Mpad / kR;
  const int per_member = std::max(1, std::min(ntiles, (sms + members - 1) / members));
  MlpTcArgs a{ntiles, Mpad, D, nsp, P, offb1, offb2, offw3, offb3, w, wimg, ximg, tile_sp64,
              y, gx, flags};
  cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kMlpSmem);
  k_mlp_tc<<<dim3(per_member, members), 128, kMlpSmem, st>>>(a);
}

}  // namespace gapgb
