// mlp_gemm_tc.cu - the surrogate's training GEMMs on the 5th-generation
// tensor cores.
//
//   C[z] = beta C[z] + A[z] B[z]^T,   A: M x K,  B: N x K,  BF16 operands,
//   FP32 accumulation in tensor memory, FP32 C (row-major, leading dim ldc)
//
// with the strided operand view of mlp.cu's SIMT GEMM: opA(m,k) =
// A[z zA + m sAm + k sAk], opB(n,k) = B[z zB + sp sBsp + n sBn + k sBk] (sp the
// species of the row tile from tile_sp, 0 without a table).  Each operand is
// either K-contiguous (sAk = 1: the forward, tangent and input-gradient
// passes) or row-contiguous (sAm = 1: the weight gradients, A = zbar^T,
// B = a^T, whose K is the batch of rows).
//
// One CTA (4 warps, thread = tile row) owns a 128-row tile of C and all of
// its N <= 128 columns.  K runs in chunks of 64 through two shared-memory
// stages: the 128 threads load chunk c + 1 with plain 16-byte loads, writing
// the no-swizzle K-major canonical layout (8-row x 16-byte core matrices,
// K-adjacent cores 128 B apart, 8-row groups 1 KB apart; row-contiguous
// operands are transposed on the way), while one thread's four
// tcgen05.mma (M 128, K 16) of chunk c run.  A stage is refilled only after
// the tcgen05.commit of the MMAs that read it has arrived; every mbarrier wait
// is bounded (a wait that gives up raises the timeout flag, and the CTA
// frees its tensor memory and returns).  The epilogue reads the accumulator
// with tcgen05.ld, thread = row.
//
// A launch with few row tiles (the weight gradients: one 128-row tile per
// (member, species) block, K = the batch's rows) splits K over CTAs: CTA x of
// a tile takes chunks [x ks, (x + 1) ks), writes its partial product to a
// scratch array, and a second kernel adds the partials in split order (so
// the result does not depend on scheduling) into C.
//
// Row tiles follow mlp.cu's species segments, which are padded to 128 rows:
// a 128-row tile lies in one segment, and a tile whose table entries are
// both negative (padding) is skipped, as the SIMT kernel skips its 64-row
// padding tiles.
#include <cuda_bf16.h>

#include <algorithm>

#include "gapgb_internal.h"
#include "tc_util.cuh"

namespace gapgb {
namespace {

using namespace tc;

constexpr int kGM = 128;                  // rows per CTA (UMMA M)
constexpr int kGK = 64;                   // K per stage
constexpr int kGA = kGM * kGK * 2;        // A stage: 16 KB
constexpr int kGB = 128 * kGK * 2;        // B stage (N <= 128): 16 KB
constexpr int kGStage = kGA + kGB;
constexpr int kGOffBar = 2 * kGStage;     // two stages, then the barriers
constexpr int kGSmem = kGOffBar + 64 + 1024;  // + alignment slack

// one operand chunk (rows [r0, r0 + rows), K [k0, k0 + 64)) into a stage in
// the K-major canonical layout, zero outside [0, nrows) x [0, K)
// (s_row, s_k: the operand's strides; s_k == 1 is K-contiguous, otherwise
// s_row == 1, row-contiguous)
__device__ __forceinline__ void load_chunk(unsigned char *dst, const __nv_bfloat16 *src,
                                           int s_row, int s_k, int r0, int nrows, int rows,
                                           int k0, int K, int tid) {
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  if (s_k == 1) {
    // 16-byte pieces along K: piece p = (row, 8-wide K group)
    for (int p = tid; p < rows * (kGK / 8); p += 128) {
      const int r = p / (kGK / 8), g = p % (kGK / 8);
      const int row = r0 + r, k = k0 + g * 8;
      uint4 v = zero;
      if (row < nrows && k < K)  // K is a multiple of 8 (checked by the launcher)
        v = *reinterpret_cast<const uint4 *>(src + (size_t)row * s_row + k);
      *reinterpret_cast<uint4 *>(dst + kmajor_off(r, g * 8, kGK / 8)) = v;
    }
  } else {
    // 16-byte pieces along the rows (s_row = 1): piece p = (k, 8-wide row group),
    // transposed into eight 2-byte stores
    for (int p = tid; p < kGK * (rows / 8); p += 128) {
      const int kk = p / (rows / 8), g = p % (rows / 8);
      const int row = r0 + g * 8, k = k0 + kk;
      uint4 v = zero;
      if (row < nrows && k < K)  // nrows is a multiple of 8 (checked by the launcher)
        v = *reinterpret_cast<const uint4 *>(src + (size_t)k * s_k + row);
      const unsigned short *h = reinterpret_cast<const unsigned short *>(&v);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        *reinterpret_cast<unsigned short *>(dst + kmajor_off(g * 8 + q, kk, kGK / 8)) = h[q];
    }
  }
}

template <int BN>
__global__ void __launch_bounds__(128)
    k_mlp_gemm_tc(int M, int N, int K, const __nv_bfloat16 *__restrict__ A, int sAm, int sAk,
                  size_t zA, const __nv_bfloat16 *__restrict__ B, int sBn, int sBk, size_t zB,
                  const int *__restrict__ tile_sp, size_t sBsp, float *__restrict__ C, int ldc,
                  size_t zC, float beta, int *__restrict__ flags, int ks,
                  float *__restrict__ part) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kGM;
  // the tile's two 64-row halves: their species, or negative for padding
  int sp0 = 0, sp1 = 0;
  if (tile_sp) {
    sp0 = tile_sp[2 * blockIdx.y];
    sp1 = (m0 + 64 < M) ? tile_sp[2 * blockIdx.y + 1] : -1;
    if (sp0 < 0 && sp1 < 0) return;
  }
  const int sp = sp0 >= 0 ? sp0 : sp1;
  A += blockIdx.z * zA;
  B += blockIdx.z * zB + (size_t)sp * sBsp;
  C += blockIdx.z * zC;
  const uint32_t s_base = smem_u32(sm);
  const uint32_t bar0 = s_base + kGOffBar, bar1 = bar0 + 8;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + kGOffBar + 16);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "n"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = instr_desc(kGM, BN);
  // this CTA's chunks of K: all of them, or split x's run of ks
  const int nk_all = (K + kGK - 1) / kGK;
  const int cb = part ? blockIdx.x * ks : 0;
  const int nk = part ? min(ks, nk_all - cb) : nk_all;
  bool ok = true;
  int waited[2] = {0, 0};  // commits of each stage waited for
  int issued[2] = {0, 0};  // commits of each stage issued
  for (int c = 0; c < nk && ok; ++c) {
    const int s = c & 1;
    // the stage's previous MMAs (chunk c - 2) must have read it
    if (issued[s] > waited[s]) {
      ok = mbar_wait(s ? bar1 : bar0, (uint32_t)(waited[s] & 1), flags);
      ++waited[s];
    }
    if (!__syncthreads_and(ok)) break;
    unsigned char *st = sm + s * kGStage;
    load_chunk(st, A, sAm, sAk, m0, M, kGM, (cb + c) * kGK, K, tid);
    load_chunk(st + kGA, B, sBn, sBk, 0, N, BN, (cb + c) * kGK, K, tid);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = s_base + s * kGStage, sb = sa + kGA;
#pragma unroll
      for (int kk = 0; kk < kGK / 16; ++kk) {
        const uint64_t ad = smem_desc(sa + kk * 256, 128, (kGK / 8) * 128);
        const uint64_t bd = smem_desc(sb + kk * 256, 128, (kGK / 8) * 128);
        umma(tmem, ad, bd, idesc, (c > 0 || kk > 0) ? 1u : 0u);
      }
      umma_commit(s ? bar1 : bar0);
    }
    ++issued[s];
  }
  // every MMA is done once the last commit of each stage has arrived
  for (int s = 0; s < 2; ++s)
    while (issued[s] > waited[s]) {
      const bool w = mbar_wait(s ? bar1 : bar0, (uint32_t)(waited[s] & 1), flags);
      ok = ok && w;
      ++waited[s];
    }
  ok = __syncthreads_and(ok);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok && nk > 0) {
    const int r = warp * 32 + lane, m = m0 + r;
    const bool live = m < M && (!tile_sp || (r < 64 ? sp0 : sp1) >= 0);
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      float v[32];
      tmem_ld32(tmem + lane_base + c0, v);
      if (live && part) {
        // partial [z][split][m][n] of the whole (padded-free) M x N product
        float *prow = part + (((size_t)blockIdx.z * gridDim.x + blockIdx.x) * M + m) * N;
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (c0 + j < N) prow[c0 + j] = v[j];
      } else if (live) {
        float *crow = C + (size_t)m * ldc;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int n = c0 + j;
          if (n < N) crow[n] = (beta == 0.f ? 0.f : beta * crow[n]) + v[j];
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(BN)
                 : "memory");
}

// C[z][m][n] = beta C + sum over splits (in order) of the partials
__global__ void k_mlp_splitk_reduce(int Z, int M, int N, int splits, const float *__restrict__ part,
                                    float *__restrict__ C, int ldc, size_t zC, float beta) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t mn = (size_t)M * N;
  if (t >= (size_t)Z * mn) return;
  const int z = (int)(t / mn);
  const size_t r = t % mn;
  const int m = (int)(r / N), n = (int)(r % N);
  const float *p = part + (size_t)z * splits * mn + r;
  float acc = p[0];
  for (int x = 1; x < splits; ++x) acc += p[(size_t)x * mn];
  float *c = C + z * zC + (size_t)m * ldc + n;
  *c = (beta == 0.f ? 0.f : beta * *c) + acc;
}

}  // namespace

bool mlp_gemm_tc(cudaStream_t st, int Z, int M, int N, int K, const __nv_bfloat16 *A, int sAm,
                 int sAk, size_t zA, const __nv_bfloat16 *B, int sBn, int sBk, size_t zB,
                 const int *tile_sp, size_t sBsp, float *C, int ldc, size_t zC, float beta,
                 int *flags, float *part, size_t part_elems) {
  // shapes and strides the staging covers: N <= 128 in one tile, each operand
  // K-contiguous with 16-byte rows or row-contiguous with 16-byte K rows,
  // 16-byte aligned bases and batch offsets
  auto al16 = [](const void *p) { return ((uintptr_t)p & 15) == 0; };
  auto mult8 = [](size_t v) { return v % 8 == 0; };
  if (N <= 0 || N > 128 || M <= 0 || K <= 0 || Z <= 0 || !flags) return false;
  if (!al16(A) || !al16(B)) return false;
  if (!mult8(zA) || !mult8(zB) || !mult8(sBsp)) return false;
  const bool a_k = sAk == 1 && mult8((size_t)sAm) && K % 8 == 0;
  const bool a_m = sAm == 1 && mult8((size_t)sAk) && M % 8 == 0;
  const bool b_k = sBk == 1 && mult8((size_t)sBn) && K % 8 == 0;
  const bool b_n = sBn == 1 && mult8((size_t)sBk) && N % 8 == 0;
  if (!(a_k || a_m) || !(b_k || b_n)) return false;
  // split K when the row tiles alone would leave most SMs idle (at least
  // two chunks per split, about two CTAs per SM, within the scratch)
  const int mt = (M + kGM - 1) / kGM, nk = (K + kGK - 1) / kGK;
  int splits = 1, ks = nk;
  if (part && !tile_sp && mt * Z < device_sms() && nk >= 4) {
    splits = std::min(nk / 2, (2 * device_sms() + mt * Z - 1) / (mt * Z));
    while (splits > 1 && (size_t)Z * splits * M * N > part_elems) --splits;
    ks = (nk + splits - 1) / splits;
    splits = (nk + ks - 1) / ks;
  }
  float *pp = splits > 1 ? part : nullptr;
  const dim3 grid(splits, mt, Z);
  if (N <= 64) {
    kernel_smem((const void *)k_mlp_gemm_tc<64>, kGSmem, true);
    k_mlp_gemm_tc<64><<<grid, 128, kGSmem, st>>>(M, N, K, A, sAm, sAk, zA, B, sBn, sBk, zB,
                                                  tile_sp, sBsp, C, ldc, zC, beta, flags, ks, pp);
  } else {
    kernel_smem((const void *)k_mlp_gemm_tc<128>, kGSmem, true);
    k_mlp_gemm_tc<128><<<grid, 128, kGSmem, st>>>(M, N, K, A, sAm, sAk, zA, B, sBn, sBk, zB,
                                                   tile_sp, sBsp, C, ldc, zC, beta, flags, ks, pp);
  }
  if (pp) {
    const size_t n = (size_t)Z * M * N;
    k_mlp_splitk_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(Z, M, N, splits, pp, C, ldc,
                                                                      zC, beta);
  }
  return true;
}

}  // namespace gapgb
