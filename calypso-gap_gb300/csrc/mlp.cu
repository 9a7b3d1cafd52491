// mlp.cu - the learned surrogate: a committee of per-species MLPs over the
// wACSF descriptors, trained on the GAP's own atomic energies and dE/dG with
// hand-written forward, backward and Adam kernels, and evaluated with the
// exact GPR as fallback for atoms the committee disagrees on.  There is no
// counterpart in the reference (gappy evaluates the GPR only).
//
// Network of one (member q, species s) block, normalised units:
//   x  = (G - mu) / sd                     standardised descriptor (BF16)
//   z1 = W1 x + b1,   a1 = silu(z1)        W1: H x D (BF16), b1 (FP32)
//   z2 = W2 a1 + b2,  a2 = silu(z2)        W2: H x H (BF16), b2 (FP32)
//   y  = w3 . a2 + b3                      w3, b3 (FP32)
//   e  = e_scale * y + e_shift[s]          atomic energy (eV)
// Input gradient: d2 = w3 o silu'(z2), d1 = silu'(z1) o (W2^T d2),
//   g = W1^T d1 (dy/dx),  dE/dG = e_scale * g / sd.
// Training loss over a batch of B rows of one block, with the labels
// normalised the same way (y* = (e* - e_shift) / e_scale, t* = dE*/dG * sd /
// e_scale):  L = (1/B) sum_b (y_b - y*_b)^2 + lambda |g_b - t*_b|^2.
// Forces are the fixed linear map F = -J^T dE/dG of the descriptor
// gradient, so matching dE/dG per atom is the force term of the loss.
// Its weight gradient (double backpropagation): with eps_b = 2 (y_b - y*_b)/B
// and r_b = 2 lambda (g_b - t*_b) / B,
//   dL/dtheta = sum_b eps_b dy_b/dtheta + d(r_b . g_b)/dtheta,
// and r . g is the directional derivative of y along r: a tangent pass
//   u1 = W1 r, v1 = silu'(z1) o u1, u2 = W2 v1, v2 = silu'(z2) o u2, r.g = w3.v2
// followed by one reverse pass over the value and the tangent:
//   zbar2 = eps w3 o silu'(z2) + w3 o silu''(z2) o u2,  ubar2 = w3 o silu'(z2)
//   dW2 = zbar2 a1^T + ubar2 v1^T,  db2 = zbar2,  dw3 = eps a2 + v2,  db3 = eps
//   abar1 = W2^T zbar2,  vbar1 = W2^T ubar2
//   zbar1 = abar1 o silu'(z1) + vbar1 o silu''(z1) o u1,  ubar1 = vbar1 o silu'(z1)
//   dW1 = zbar1 x^T + ubar1 r^T,  db1 = zbar1.
// Precision: FP32 master weights and Adam moments; BF16 copies of W1 and W2
// and BF16 row operands (x, a1, r, v1, zbar, ubar) feed the GEMMs, which
// accumulate in FP32; all other intermediates are FP32.
//
// Batching: every GEMM runs all committee members (blockIdx.z) and all
// species at once.  Rows are laid out in species segments padded to the
// 64-row tile, and each row tile reads its weight block through a
// tile -> species table, so one launch covers a mixed-species batch.
// Training draws the same number R of rows per species for every member
// (segment z = q * nspecies + s holds rows [z R, (z + 1) R)); prediction
// partitions the atoms by species on the device, so its launch shapes depend
// only on the atom count and it can be captured in a CUDA graph.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <type_traits>
#include <vector>

#include "gapgb_internal.h"

namespace gapgb {
namespace {

constexpr int kTile = 64;      // rows per SIMT GEMM tile
constexpr int kSeg = 128;      // species segments are padded to the tensor-core tile
constexpr int kMaxSurrSpecies = 16;

__device__ __forceinline__ float ldf(const float *p, size_t i) { return p[i]; }
__device__ __forceinline__ float ldf(const __nv_bfloat16 *p, size_t i) {
  return __bfloat162float(p[i]);
}

// C[z][m][n] = beta C + sum_k opA(m,k) opB(n,k), opA(m,k) = A[z zA + m sAm + k sAk],
// opB(n,k) = B[z zB + sp sBsp + n sBn + k sBk] with sp = tile_sp[m-tile] (0 when
// tile_sp is null).  Row tiles whose tile_sp entry is negative are padding and
// are skipped.  64 x 64 output tile per block, 4 x 4 per thread.
template <typename TA, typename TB>
__global__ void __launch_bounds__(256)
    k_mlp_gemm(int M, int N, int K, const TA *__restrict__ A, int sAm, int sAk, size_t zA,
               const TB *__restrict__ B, int sBn, int sBk, size_t zB, const int *__restrict__ tile_sp,
               size_t sBsp, float *__restrict__ C, int ldc, size_t zC, float beta) {
  __shared__ float As[16][kTile + 4];
  __shared__ float Bs[16][kTile + 4];
  int sp = 0;
  if (tile_sp) {
    sp = tile_sp[blockIdx.y];
    if (sp < 0) return;
  }
  A += blockIdx.z * zA;
  B += blockIdx.z * zB + sp * sBsp;
  C += blockIdx.z * zC;
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  const bool a_kfast = sAk == 1, b_kfast = sBk == 1;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int q = t; q < kTile * 16; q += 256) {
      // consecutive threads walk the unit-stride dimension of each operand
      int r = a_kfast ? q >> 4 : q & 63, kk = a_kfast ? q & 15 : q >> 6;
      int m = m0 + r, k = k0 + kk;
      As[kk][r] = (m < M && k < K) ? ldf(A, (size_t)m * sAm + (size_t)k * sAk) : 0.f;
      r = b_kfast ? q >> 4 : q & 63;
      kk = b_kfast ? q & 15 : q >> 6;
      const int n = n0 + r;
      k = k0 + kk;
      Bs[kk][r] = (n < N && k < K) ? ldf(B, (size_t)n * sBn + (size_t)k * sBk) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
      if (m < M && n < N) {
        float *c = C + (size_t)m * ldc + n;
        *c = (beta == 0.f ? 0.f : beta * *c) + acc[i][j];
      }
    }
}

// logistic function with the fast reciprocal (2-ulp division): the values
// feed BF16 operands or FP32 sums where that error is far below the rest
__device__ __forceinline__ float sigm(float z) { return __fdividef(1.f, 1.f + __expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = sigm(z);
  return s * (1.f + z * (1.f - s));
}
__device__ __forceinline__ float d2silu(float z) {
  const float s = sigm(z);
  return s * (1.f - s) * (2.f + z * (1.f - 2.f * s));
}

// Row r of a [members][rows][.] buffer: member q = r / rows, species from the
// row's tile.  Parameter block of (q, sp): w + (q * nsp + sp) * P.
struct RowMap {
  int rows, nsp;
  size_t P;
  const int *tile_sp;
  __device__ int species(int row_in_member) const { return tile_sp[row_in_member / kTile]; }
};

// x = (G[idx] - mu) * isig as BF16 for every row (idx < 0: padding, zeros)
__global__ void k_mlp_gather(size_t nrows, int D, const int *__restrict__ idx,
                             const float *__restrict__ G, const float *__restrict__ mu,
                             const float *__restrict__ isig, __nv_bfloat16 *__restrict__ X) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows * D) return;
  const size_t r = i / D;
  const int d = (int)(i - r * D);
  const int a = idx[r];
  X[i] = __float2bfloat16(a >= 0 ? (G[(size_t)a * D + d] - mu[d]) * isig[d] : 0.f);
}

// Z += bias (per row species), A = silu(Z) in BF16 when A is non-null
__global__ void k_mlp_bias_act(RowMap rm, int members, int H, size_t boff, const float *__restrict__ w,
                               float *__restrict__ Z, __nv_bfloat16 *__restrict__ A) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t per = (size_t)rm.rows * H;
  if (i >= per * members) return;
  const int q = (int)(i / per);
  const size_t rr = i - (size_t)q * per;
  const int row = (int)(rr / H), h = (int)(rr - (size_t)row * H);
  const int sp = rm.species(row);
  if (sp < 0) return;
  const float z = Z[i] + w[(size_t)(q * rm.nsp + sp) * rm.P + boff + h];
  Z[i] = z;
  if (A) A[i] = __float2bfloat16(silu(z));
}

// y = w3 . silu(z2) + b3 and D2 = w3 o silu'(z2) (one warp per row)
__global__ void k_mlp_out(RowMap rm, int members, int H, size_t w3off, size_t b3off,
                          const float *__restrict__ w, const float *__restrict__ Z2,
                          float *__restrict__ y, float *__restrict__ D2) {
  const size_t row = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= (size_t)rm.rows * members) return;
  const int q = (int)(row / rm.rows), rin = (int)(row - (size_t)q * rm.rows);
  const int sp = rm.species(rin);
  if (sp < 0) return;
  const float *blk = w + (size_t)(q * rm.nsp + sp) * rm.P;
  float s = 0.f;
  for (int h = lane; h < H; h += 32) {
    const float z = Z2[row * H + h];
    s = fmaf(silu(z), blk[w3off + h], s);
    if (D2) D2[row * H + h] = blk[w3off + h] * dsilu(z);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) y[row] = s + blk[b3off];
}

// out = silu'(Z) o in; FP32 and/or BF16 outputs
__global__ void k_mlp_dsilu(size_t n, const float *__restrict__ Z, const float *in, float *out,
                            __nv_bfloat16 *__restrict__ out16) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float v = dsilu(Z[i]) * in[i];
  if (out) out[i] = v;
  if (out16) out16[i] = __float2bfloat16(v);
}

struct LossArgs {
  int R, nsp, D;
  float lambda, inv_es;
  const int *idx;
  const float *y, *g;
  const double *e_lab;
  const float *t_lab, *sd, *e_shift;
  float *eps, *Rv;
  __nv_bfloat16 *R16;
  double *loss_rows;
};

// eps = 2 (y - y*) / R, r = 2 lambda (g - t*) / R, per-row loss (one warp per row)
__global__ void k_mlp_loss(LossArgs a, size_t nrows) {
  const size_t row = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= nrows) return;
  const int at = a.idx[row];
  const int sp = (int)((row / a.R) % a.nsp);
  double lg = 0.0;
  for (int d = lane; d < a.D; d += 32) {
    const float tn = a.t_lab[(size_t)at * a.D + d] * a.sd[d] * a.inv_es;
    const float diff = a.g[row * a.D + d] - tn;
    lg += (double)diff * diff;
    const float r = 2.f * a.lambda * diff / (float)a.R;
    a.Rv[row * a.D + d] = r;
    a.R16[row * a.D + d] = __float2bfloat16(r);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) lg += __shfl_xor_sync(0xffffffffu, lg, off);
  if (lane == 0) {
    const double yl = (a.e_lab[at] - (double)a.e_shift[sp]) * (double)a.inv_es;
    const double dy = (double)a.y[row] - yl;
    a.eps[row] = (float)(2.0 * dy / a.R);
    a.loss_rows[row] = dy * dy + (double)a.lambda * lg;
  }
}

// layer-2 reverse: zbar2, ubar2 (BF16)
__global__ void k_mlp_back2(RowMap rm, int members, int H, size_t w3off, const float *__restrict__ w,
                            const float *__restrict__ Z2, const float *__restrict__ U2,
                            const float *__restrict__ eps, __nv_bfloat16 *__restrict__ Zb2,
                            __nv_bfloat16 *__restrict__ Ub2) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t per = (size_t)rm.rows * H;
  if (i >= per * members) return;
  const int q = (int)(i / per);
  const size_t rr = i - (size_t)q * per;
  const int row = (int)(rr / H), h = (int)(rr - (size_t)row * H);
  const int sp = rm.species(row);
  const float w3 = w[(size_t)(q * rm.nsp + sp) * rm.P + w3off + h];
  const float z = Z2[i];
  const float ds = dsilu(z);
  Zb2[i] = __float2bfloat16(eps[(size_t)q * rm.rows + row] * w3 * ds + w3 * d2silu(z) * U2[i]);
  Ub2[i] = __float2bfloat16(w3 * ds);
}

// layer-1 reverse: zbar1, ubar1 (BF16)
__global__ void k_mlp_back1(size_t n, const float *__restrict__ Z1, const float *__restrict__ U1,
                            const float *__restrict__ Ab1, const float *__restrict__ Vb1,
                            __nv_bfloat16 *__restrict__ Zb1, __nv_bfloat16 *__restrict__ Ub1) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float z = Z1[i], ds = dsilu(z);
  Zb1[i] = __float2bfloat16(Ab1[i] * ds + Vb1[i] * d2silu(z) * U1[i]);
  Ub1[i] = __float2bfloat16(Vb1[i] * ds);
}

// bias gradients: out[z P + off + h] = sum over the R rows of segment z
__global__ void k_mlp_colsum(int R, int H, size_t P, size_t off, const __nv_bfloat16 *__restrict__ X,
                             float *__restrict__ grad) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x, z = blockIdx.y;
  if (h >= H) return;
  const __nv_bfloat16 *x = X + (size_t)z * R * H;
  float s = 0.f;
  for (int r = 0; r < R; ++r) s += __bfloat162float(x[(size_t)r * H + h]);
  grad[(size_t)z * P + off + h] = s;
}

// dw3 = sum eps a2 + v2 and db3 = sum eps per segment
__global__ void k_mlp_grad_w3(int R, int H, size_t P, size_t w3off, size_t b3off,
                              const float *__restrict__ Z2, const float *__restrict__ U2,
                              const float *__restrict__ eps, float *__restrict__ grad) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x, z = blockIdx.y;
  const size_t r0 = (size_t)z * R;
  if (h < H) {
    float s = 0.f;
    for (int r = 0; r < R; ++r) {
      const float zz = Z2[(r0 + r) * H + h];
      s += eps[r0 + r] * silu(zz) + dsilu(zz) * U2[(r0 + r) * H + h];
    }
    grad[(size_t)z * P + w3off + h] = s;
  }
  if (h == 0) {
    float s = 0.f;
    for (int r = 0; r < R; ++r) s += eps[r0 + r];
    grad[(size_t)z * P + b3off] = s;
  }
}

// Adam with bias correction on the FP32 master weights; BF16 copy refreshed
__global__ void k_mlp_adam(size_t n, float *__restrict__ w, __nv_bfloat16 *__restrict__ w16,
                           float *__restrict__ m, float *__restrict__ v, const float *__restrict__ g,
                           float lr, float b1, float b2, float eps, float c1, float c2) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  w16[i] = __float2bfloat16(wi);
}

// ---- prediction: device-side partition of the atoms by species -----------

// per atom: surrogate species index (-1 if absent) and its slot in the segment
__global__ void k_mlp_count(int N, const int *__restrict__ Z, int nsp, const int *__restrict__ zt,
                            int *__restrict__ cnt, int *__restrict__ sp_of, int *__restrict__ slot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int sp = -1;
  for (int s = 0; s < nsp; ++s)
    if (zt[s] == Z[i]) sp = s;
  sp_of[i] = sp;
  slot[i] = sp >= 0 ? atomicAdd(&cnt[sp], 1) : -1;
}

// padded segment offsets and the tile -> species table (single block)
__global__ void k_mlp_segments(int nsp, int ntiles, const int *__restrict__ cnt, int *__restrict__ seg,
                               int *__restrict__ tile_sp) {
  __shared__ int off[kMaxSurrSpecies + 1];
  if (threadIdx.x == 0) {
    off[0] = 0;
    for (int s = 0; s < nsp; ++s) off[s + 1] = off[s] + (cnt[s] + kSeg - 1) / kSeg * kSeg;
    for (int s = 0; s <= nsp; ++s) seg[s] = off[s];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
    int sp = -1;
    for (int s = 0; s < nsp; ++s)
      if (t * kTile >= off[s] && t * kTile < off[s + 1]) sp = s;
    tile_sp[t] = sp;
  }
}

__global__ void k_mlp_scatter(int N, const int *__restrict__ sp_of, const int *__restrict__ slot,
                              const int *__restrict__ seg, int *__restrict__ idx,
                              int *__restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int sp = sp_of[i];
  if (sp < 0) {
    atomicOr(err, kFlagUnknownSpecies);
    return;
  }
  idx[seg[sp] + slot[i]] = i;
}

// committee mean / std / mean dE/dG, scattered to atom order (one warp per row)
__global__ void k_mlp_committee(int Mpad, int D, int members, const int *__restrict__ idx,
                                const int *__restrict__ tile_sp, const float *__restrict__ y,
                                const float *__restrict__ g, const float *__restrict__ isig,
                                const float *__restrict__ e_shift, float e_scale,
                                double *__restrict__ e_out, float *__restrict__ std_out,
                                float *__restrict__ dedg_out, float *__restrict__ gstd_out) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= Mpad) return;  // warp-uniform: a warp owns one row
  const int a = idx[row];
  if (a < 0) return;
  const int sp = tile_sp[row / kTile];
  const float sc = e_scale / members;
  // mean dE/dG, and the members' spread of it: |std_q(dE/dG_q)| over the D
  // components, in eV per descriptor unit (member q's dE/dG_d is
  // g_qd e_scale isig_d)
  float spread = 0.f;
  for (int d = lane; d < D; d += 32) {
    float s = 0.f;
    for (int q = 0; q < members; ++q) s += g[((size_t)q * Mpad + row) * D + d];
    dedg_out[(size_t)a * D + d] = s * sc * isig[d];
    if (gstd_out) {  // two passes: no cancellation when the members agree closely
      const float mean = __fdividef(s, (float)members);
      float var = 0.f;
      for (int q = 0; q < members; ++q) {
        const float dv = g[((size_t)q * Mpad + row) * D + d] - mean;
        var = fmaf(dv, dv, var);
      }
      spread = fmaf(isig[d] * isig[d], var / (float)(members > 1 ? members - 1 : 1), spread);
    }
  }
  if (gstd_out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) spread += __shfl_xor_sync(0xffffffffu, spread, o);
    if (lane == 0) gstd_out[a] = e_scale * sqrtf(spread);
  }
  if (lane == 0) {
    // FP32 statistics (the FP64 pipe is narrow); the energy itself in FP64
    float mean = 0.f;
    for (int q = 0; q < members; ++q) mean += y[(size_t)q * Mpad + row];
    mean = __fdividef(mean, (float)members);
    float var = 0.f;
    for (int q = 0; q < members; ++q) {
      const float dv = y[(size_t)q * Mpad + row] - mean;
      var = fmaf(dv, dv, var);
    }
    e_out[a] = (double)e_scale * (double)mean + (double)e_shift[sp];
    std_out[a] = e_scale * sqrtf(__fdividef(var, (float)(members > 1 ? members - 1 : 1)));
  }
}

// atom i takes the GPR when its committee std is above thr (or NaN), when
// the members' dE/dG spread is above gthr (> 0), or when a neighbour slot
// lies closer than r_contact (FP32 records, .w = distance)
__global__ void k_mlp_fallback(int N, const float *__restrict__ sd, float thr,
                               const float *__restrict__ gsd, float gthr,
                               const int *__restrict__ cnt, const float4 *__restrict__ d32,
                               int cap, float rcon, int *__restrict__ rows,
                               int *__restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  bool fb = !(sd[i] <= thr) || (gthr > 0.f && !(gsd[i] <= gthr));
  if (!fb && rcon > 0.f) {
    const int P = min(cnt[i], cap);
    for (int q = 0; q < P && !fb; ++q) fb = d32[(size_t)i * cap + q].w < rcon;
  }
  if (fb) rows[atomicAdd(count, 1)] = i;
}

unsigned nblk(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace
}  // namespace gapgb

using namespace gapgb;

struct gapgb_surrogate {
  int nsp = 0, D = 0, H = 0, members = 0;
  std::vector<int> species_z;
  size_t P = 0;  // parameters per (member, species) block
  size_t W1 = 0, b1 = 0, W2 = 0, b2 = 0, w3 = 0, b3 = 0;
  float *w = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
  int *t_err = nullptr;  // error flags of the training GEMMs (bounded tensor-core waits)
  float *t_part = nullptr;  // split-K partials of the weight-gradient GEMMs
  size_t t_part_n = 0;
  __nv_bfloat16 *w16 = nullptr;
  float *mu = nullptr, *isig = nullptr, *sd = nullptr, *e_shift = nullptr;
  int *zt = nullptr;
  float e_scale = 1.f;
  long step = 0;
  int device = 0;
  // training tile table (rows_per_species R)
  int train_R = 0;
  int *t_tile_sp = nullptr;
  // activation buffers, sized for `cap_rows` rows over all members
  size_t cap_rows = 0;
  __nv_bfloat16 *X = nullptr, *A1 = nullptr, *R16 = nullptr, *V1 = nullptr, *Zb2 = nullptr,
                *Ub2 = nullptr, *Zb1 = nullptr, *Ub1 = nullptr;
  float *Z1 = nullptr, *Z2 = nullptr, *D2 = nullptr, *D1 = nullptr, *Gx = nullptr, *y = nullptr,
        *eps = nullptr, *Rv = nullptr, *U1 = nullptr, *U2 = nullptr, *Ab1 = nullptr, *Vb1 = nullptr;
  int *idx = nullptr;
  double *lrows = nullptr;
  // prediction partition (sized for `cap_atoms`)
  int cap_atoms = 0, cap_tiles = 0;
  unsigned char *w_img = nullptr;  // tensor-core weight images
  unsigned char *x_img = nullptr;  // tensor-core row tiles (cap_tiles * 64 rows)
  int *p_cnt = nullptr, *p_sp = nullptr, *p_slot = nullptr, *p_seg = nullptr, *p_tile = nullptr,
      *p_err = nullptr;
  cudaStream_t stream = nullptr;
};

namespace {

gapgb_status sfail(gapgb_status st, const std::string &msg) {
  set_last_error(msg);
  return st;
}

// tc_flags: the error flags of the tensor-core form (mlp_gemm_tc.cu), which
// takes BF16 x BF16 products when its shape and stride rules hold; null keeps
// the SIMT kernel (FP32 operands, or row tiles that may straddle species)
template <typename TA, typename TB>
void gemm(cudaStream_t st, int Z, int M, int N, int K, const TA *A, int sAm, int sAk, size_t zA,
          const TB *B, int sBn, int sBk, size_t zB, const int *tile_sp, size_t sBsp, float *C,
          int ldc, size_t zC, float beta, int *tc_flags = nullptr, float *tc_part = nullptr,
          size_t tc_part_n = 0) {
  if constexpr (std::is_same<TA, __nv_bfloat16>::value && std::is_same<TB, __nv_bfloat16>::value) {
    if (tc_flags && mlp_gemm_tc(st, Z, M, N, K, A, sAm, sAk, zA, B, sBn, sBk, zB, tile_sp, sBsp,
                                C, ldc, zC, beta, tc_flags, tc_part, tc_part_n))
      return;
  }
  dim3 g((N + kTile - 1) / kTile, (M + kTile - 1) / kTile, Z);
  k_mlp_gemm<TA, TB><<<g, 256, 0, st>>>(M, N, K, A, sAm, sAk, zA, B, sBn, sBk, zB, tile_sp, sBsp, C,
                                        ldc, zC, beta);
}

template <typename T>
bool dalloc(T **p, size_t n) {
  return cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T)) == cudaSuccess;
}

void free_rows(gapgb_surrogate *s) {
  void *ps[] = {s->X, s->A1, s->R16, s->V1, s->Zb2, s->Ub2, s->Zb1, s->Ub1, s->Z1, s->Z2, s->D2,
                s->D1, s->Gx, s->y, s->eps, s->Rv, s->U1, s->U2, s->Ab1, s->Vb1, s->idx, s->lrows};
  for (void *p : ps)
    if (p) cudaFree(p);
  s->X = s->A1 = s->R16 = s->V1 = s->Zb2 = s->Ub2 = s->Zb1 = s->Ub1 = nullptr;
  s->Z1 = s->Z2 = s->D2 = s->D1 = s->Gx = s->y = s->eps = s->Rv = s->U1 = s->U2 = s->Ab1 = s->Vb1 =
      nullptr;
  s->idx = nullptr;
  s->lrows = nullptr;
  s->cap_rows = 0;
}

// activation buffers for `rows` rows over all members
gapgb_status ensure_rows(gapgb_surrogate *s, size_t rows) {
  if (rows <= s->cap_rows) return GAPGB_OK;
  free_rows(s);
  const size_t W = rows * std::max(s->D, s->H);
  bool ok = dalloc(&s->X, W) && dalloc(&s->A1, W) && dalloc(&s->R16, W) && dalloc(&s->V1, W) &&
            dalloc(&s->Zb2, W) && dalloc(&s->Ub2, W) && dalloc(&s->Zb1, W) && dalloc(&s->Ub1, W) &&
            dalloc(&s->Z1, W) && dalloc(&s->Z2, W) && dalloc(&s->D2, W) && dalloc(&s->D1, W) &&
            dalloc(&s->Gx, W) && dalloc(&s->y, rows) && dalloc(&s->eps, rows) && dalloc(&s->Rv, W) &&
            dalloc(&s->U1, W) && dalloc(&s->U2, W) && dalloc(&s->Ab1, W) && dalloc(&s->Vb1, W) &&
            dalloc(&s->idx, rows) && dalloc(&s->lrows, rows);
  if (!ok) {
    free_rows(s);
    cudaGetLastError();
    return sfail(GAPGB_ERR_ALLOC, "surrogate activation buffers");
  }
  s->cap_rows = rows;
  return GAPGB_OK;
}

// 64-row tiles of the species-sorted rows (segments padded to 128 rows)
int pad_tiles(int N, int nsp) {
  return (N + nsp * (kSeg - 1) + kSeg - 1) / kSeg * (kSeg / kTile);
}

gapgb_status ensure_atoms(gapgb_surrogate *s, int N) {
  const int tiles = pad_tiles(N, s->nsp);
  if (N <= s->cap_atoms && tiles <= s->cap_tiles) return GAPGB_OK;
  int *ps[] = {s->p_cnt, s->p_sp, s->p_slot, s->p_seg, s->p_tile, s->p_err};
  for (int *p : ps)
    if (p) cudaFree(p);
  if (s->x_img) cudaFree(s->x_img);
  s->p_cnt = s->p_sp = s->p_slot = s->p_seg = s->p_tile = s->p_err = nullptr;
  s->x_img = nullptr;
  s->cap_atoms = s->cap_tiles = 0;
  const bool tcx = mlp_tc_eligible(s->D, s->H);
  if (!(dalloc(&s->p_cnt, kMaxSurrSpecies) && dalloc(&s->p_sp, N) && dalloc(&s->p_slot, N) &&
        dalloc(&s->p_seg, kMaxSurrSpecies + 1) && dalloc(&s->p_tile, tiles) && dalloc(&s->p_err, 1) &&
        (!tcx || dalloc(&s->x_img, mlp_tc_x_image_bytes(tiles * kTile))))) {
    cudaGetLastError();
    return sfail(GAPGB_ERR_ALLOC, "surrogate partition buffers");
  }
  s->cap_atoms = N;
  s->cap_tiles = tiles;
  return GAPGB_OK;
}

// Forward over `rows` rows per member (s->X filled); y and, with want_grad,
// the input gradient Gx.  zX = 0 shares X across members (prediction).
void forward(gapgb_surrogate *s, cudaStream_t st, int rows, const int *tile_sp, size_t zX,
             bool want_grad, int *tc_flags = nullptr) {
  const int D = s->D, H = s->H, Q = s->members;
  const size_t mstride = (size_t)s->nsp * s->P;  // member stride of the parameters
  const size_t zH = (size_t)rows * H, zD = (size_t)rows * D;
  RowMap rm{rows, s->nsp, s->P, tile_sp};
  gemm(st, Q, rows, H, D, s->X, D, 1, zX, s->w16 + s->W1, D, 1, mstride, tile_sp, s->P, s->Z1, H, zH,
       0.f, tc_flags);
  k_mlp_bias_act<<<nblk(zH * Q), 256, 0, st>>>(rm, Q, H, s->b1, s->w, s->Z1, s->A1);
  gemm(st, Q, rows, H, H, s->A1, H, 1, zH, s->w16 + s->W2, H, 1, mstride, tile_sp, s->P, s->Z2, H, zH,
       0.f, tc_flags);
  k_mlp_bias_act<<<nblk(zH * Q), 256, 0, st>>>(rm, Q, H, s->b2, s->w, s->Z2, nullptr);
  k_mlp_out<<<nblk((size_t)rows * Q * 32), 256, 0, st>>>(rm, Q, H, s->w3, s->b3, s->w, s->Z2, s->y,
                                                         want_grad ? s->D2 : nullptr);
  if (!want_grad) return;
  // d1 = silu'(z1) o (W2^T d2): opB(n=j, k=i) = W2[i][j]
  gemm(st, Q, rows, H, H, s->D2, H, 1, zH, s->w16 + s->W2, 1, H, mstride, tile_sp, s->P, s->D1, H, zH, 0.f);
  k_mlp_dsilu<<<nblk(zH * Q), 256, 0, st>>>(zH * Q, s->Z1, s->D1, s->D1, nullptr);
  // g = W1^T d1: opB(n=d, k=h) = W1[h][d]
  gemm(st, Q, rows, D, H, s->D1, H, 1, zH, s->w16 + s->W1, 1, D, mstride, tile_sp, s->P, s->Gx, D, zD, 0.f);
}

}  // namespace

namespace gapgb {

// Buffers for a committee prediction over N atoms (allocates; call before
// any stream capture of surrogate_enqueue).
gapgb_status surrogate_prepare(gapgb_surrogate *s, int N) {
  gapgb_status st = ensure_atoms(s, N);
  if (st) return st;
  if (mlp_tc_eligible(s->D, s->H) && !s->w_img &&
      !dalloc(&s->w_img, mlp_tc_w_image_bytes(s->members * s->nsp))) {
    cudaGetLastError();
    return sfail(GAPGB_ERR_ALLOC, "surrogate weight images");
  }
  return ensure_rows(s, (size_t)s->cap_tiles * kTile * s->members);
}

// Committee prediction for N atoms (atomic numbers d_Z, FP32 descriptors
// d_G) on stream st: e (eV), committee std (eV) and mean dE/dG per atom.
// Launch shapes depend on N only; no allocation, no synchronisation.
void surrogate_enqueue(gapgb_surrogate *s, int N, const int *d_Z, const float *d_G, double *d_e,
                       float *d_std, float *d_dedg, float *d_gstd, int *d_err, cudaStream_t st) {
  const int tiles = pad_tiles(N, s->nsp);
  const int Mpad = tiles * kTile;
  cudaMemsetAsync(s->p_cnt, 0, kMaxSurrSpecies * sizeof(int), st);
  cudaMemsetAsync(s->idx, 0xff, (size_t)Mpad * sizeof(int), st);
  k_mlp_count<<<nblk(N), 256, 0, st>>>(N, d_Z, s->nsp, s->zt, s->p_cnt, s->p_sp, s->p_slot);
  k_mlp_segments<<<1, 256, 0, st>>>(s->nsp, tiles, s->p_cnt, s->p_seg, s->p_tile);
  k_mlp_scatter<<<nblk(N), 256, 0, st>>>(N, s->p_sp, s->p_slot, s->p_seg, s->idx, d_err);
  if (mlp_tc_eligible(s->D, s->H)) {
    // tensor cores: BF16 weight images from the current weights, then the
    // fused forward + input gradient of every member
    launch_mlp_w_image(s->members * s->nsp, s->D, s->P, s->W1, s->W2, s->b1, s->b2, s->w3,
                       s->b3, s->w16, s->w, s->w_img, st);
    launch_mlp_tc(s->members, s->nsp, s->D, Mpad, s->w_img, s->x_img, s->idx, d_G, s->mu,
                  s->isig, s->p_tile, s->y, s->Gx, d_err, st);
  } else {
    k_mlp_gather<<<nblk((size_t)Mpad * s->D), 256, 0, st>>>(Mpad, s->D, s->idx, d_G, s->mu,
                                                          s->isig, s->X);
    forward(s, st, Mpad, s->p_tile, 0, true);
  }
  k_mlp_committee<<<nblk((size_t)Mpad * 32), 256, 0, st>>>(Mpad, s->D, s->members, s->idx, s->p_tile,
                                                          s->y, s->Gx, s->isig, s->e_shift,
                                                          s->e_scale, d_e, d_std, d_dedg,
                                                          d_gstd);
}

int surrogate_device(const gapgb_surrogate *s) { return s->device; }
int surrogate_des_len(const gapgb_surrogate *s) { return s->D; }
bool surrogate_has_species(const gapgb_surrogate *s, int z) {
  return std::find(s->species_z.begin(), s->species_z.end(), z) != s->species_z.end();
}

// rows[0 .. *count) = atoms whose committee std is above the threshold (or
// NaN), whose dE/dG spread is above grad_spread (0: off), or that have a
// neighbour closer than r_contact (0: off)
void surrogate_select_fallback(int N, const float *d_std, float threshold, const float *d_gstd,
                               float grad_spread, const int *d_cnt, const float4 *d_d32, int cap,
                               float r_contact, int *d_rows, int *d_count, cudaStream_t st) {
  cudaMemsetAsync(d_count, 0, sizeof(int), st);
  k_mlp_fallback<<<nblk(N), 256, 0, st>>>(N, d_std, threshold, d_gstd, grad_spread, d_cnt, d_d32,
                                          cap, r_contact, d_rows, d_count);
}

}  // namespace gapgb

extern "C" {

gapgb_status gapgb_surrogate_create(int nspecies, const int *species_z, int des_len, int hidden,
                                    int members, unsigned long long seed, gapgb_surrogate **out) {
  if (!out || !species_z) return sfail(GAPGB_ERR_ARG, "null argument");
  *out = nullptr;
  if (nspecies <= 0 || nspecies > kMaxSurrSpecies || des_len <= 0 || hidden <= 0 || members <= 0)
    return sfail(GAPGB_ERR_ARG, "surrogate shape out of range (1..16 species, positive sizes)");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return sfail(GAPGB_ERR_NO_DEVICE, "no CUDA device visible");
  }
  gapgb_surrogate *s = new gapgb_surrogate();
  cudaGetDevice(&s->device);
  s->nsp = nspecies;
  s->species_z.assign(species_z, species_z + nspecies);
  s->D = des_len;
  s->H = hidden;
  s->members = members;
  s->W1 = 0;
  s->b1 = s->W1 + (size_t)hidden * des_len;
  s->W2 = s->b1 + hidden;
  s->b2 = s->W2 + (size_t)hidden * hidden;
  s->w3 = s->b2 + hidden;
  s->b3 = s->w3 + hidden;
  // blocks padded to 8 parameters, so that every block's BF16 weights start
  // on a 16-byte boundary (the tensor-core training GEMMs load 16 bytes at a
  // time); the padding stays zero
  s->P = (s->b3 + 1 + 7) / 8 * 8;
  const size_t n = (size_t)members * nspecies * s->P;
  // variance-scaled normal initialisation, an independent draw per member
  std::vector<float> w(n, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> n1(0.f, std::sqrt(1.f / des_len)), n2(0.f, std::sqrt(1.f / hidden));
  for (int z = 0; z < members * nspecies; ++z) {
    float *b = w.data() + (size_t)z * s->P;
    for (size_t i = 0; i < (size_t)hidden * des_len; ++i) b[s->W1 + i] = n1(rng);
    for (size_t i = 0; i < (size_t)hidden * hidden; ++i) b[s->W2 + i] = n2(rng);
    for (int i = 0; i < hidden; ++i) b[s->w3 + i] = n2(rng);
  }
  std::vector<__nv_bfloat16> w16(n);
  for (size_t i = 0; i < n; ++i) w16[i] = __float2bfloat16(w[i]);
  std::vector<float> zeros(std::max(des_len, kMaxSurrSpecies), 0.f), ones(des_len, 1.f);
  if (!(dalloc(&s->w, n) && dalloc(&s->m, n) && dalloc(&s->v, n) && dalloc(&s->grad, n) &&
        dalloc(&s->t_err, 1) &&
        dalloc(&s->w16, n) && dalloc(&s->mu, des_len) && dalloc(&s->isig, des_len) &&
        dalloc(&s->sd, des_len) && dalloc(&s->e_shift, kMaxSurrSpecies) && dalloc(&s->zt, nspecies))) {
    cudaGetLastError();
    gapgb_surrogate_free(s);
    return sfail(GAPGB_ERR_ALLOC, "surrogate weights");
  }
  bool ok = cudaMemcpy(s->w, w.data(), n * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(s->w16, w16.data(), n * 2, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemset(s->m, 0, n * 4) == cudaSuccess && cudaMemset(s->v, 0, n * 4) == cudaSuccess &&
            cudaMemset(s->grad, 0, n * 4) == cudaSuccess &&
            cudaMemset(s->t_err, 0, sizeof(int)) == cudaSuccess &&
            cudaMemcpy(s->mu, zeros.data(), des_len * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(s->isig, ones.data(), des_len * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(s->sd, ones.data(), des_len * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(s->e_shift, zeros.data(), kMaxSurrSpecies * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(s->zt, species_z, nspecies * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess;
  if (!ok) {
    const cudaError_t e = cudaGetLastError();
    gapgb_surrogate_free(s);
    return sfail(GAPGB_ERR_CUDA, std::string("surrogate set-up: ") + cudaGetErrorString(e));
  }
  *out = s;
  return GAPGB_OK;
}

void gapgb_surrogate_free(gapgb_surrogate *s) {
  if (!s) return;
  free_rows(s);
  void *ps[] = {s->w, s->m, s->v, s->grad, s->t_err, s->t_part, s->w16, s->mu, s->isig, s->sd, s->e_shift, s->zt,
                s->t_tile_sp, s->p_cnt, s->p_sp, s->p_slot, s->p_seg, s->p_tile, s->p_err,
                s->w_img, s->x_img};
  for (void *p : ps)
    if (p) cudaFree(p);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

gapgb_status gapgb_surrogate_info(const gapgb_surrogate *s, int *nspecies, int *des_len, int *hidden,
                                  int *members, size_t *params_per_block) {
  if (!s) return sfail(GAPGB_ERR_ARG, "null surrogate");
  if (nspecies) *nspecies = s->nsp;
  if (des_len) *des_len = s->D;
  if (hidden) *hidden = s->H;
  if (members) *members = s->members;
  if (params_per_block) *params_per_block = s->P;
  return GAPGB_OK;
}

gapgb_status gapgb_surrogate_set_norm(gapgb_surrogate *s, const double *g_mean, const double *g_std,
                                      const double *e_shift, double e_scale) {
  if (!s || !g_mean || !g_std || !e_shift) return sfail(GAPGB_ERR_ARG, "null argument");
  if (!(e_scale > 0.0)) return sfail(GAPGB_ERR_ARG, "e_scale must be positive");
  std::vector<float> mu(s->D), is(s->D), sd(s->D), sh(kMaxSurrSpecies, 0.f);
  for (int d = 0; d < s->D; ++d) {
    const bool live = g_std[d] > 1e-12;
    mu[d] = (float)g_mean[d];
    sd[d] = live ? (float)g_std[d] : 1.f;
    is[d] = live ? (float)(1.0 / g_std[d]) : 1.f;
  }
  for (int q = 0; q < s->nsp; ++q) sh[q] = (float)e_shift[q];
  s->e_scale = (float)e_scale;
  GAPGB_CUDA_TRY(cudaSetDevice(s->device));
  GAPGB_CUDA_TRY(cudaMemcpy(s->mu, mu.data(), s->D * 4, cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMemcpy(s->isig, is.data(), s->D * 4, cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMemcpy(s->sd, sd.data(), s->D * 4, cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMemcpy(s->e_shift, sh.data(), kMaxSurrSpecies * 4, cudaMemcpyHostToDevice));
  return GAPGB_OK;
}

gapgb_status gapgb_surrogate_params(gapgb_surrogate *s, float *get, const float *set) {
  if (!s) return sfail(GAPGB_ERR_ARG, "null surrogate");
  GAPGB_CUDA_TRY(cudaSetDevice(s->device));
  const size_t n = (size_t)s->members * s->nsp * s->P;
  if (get) GAPGB_CUDA_TRY(cudaMemcpy(get, s->w, n * 4, cudaMemcpyDeviceToHost));
  if (set) {
    std::vector<__nv_bfloat16> w16(n);
    for (size_t i = 0; i < n; ++i) w16[i] = __float2bfloat16(set[i]);
    GAPGB_CUDA_TRY(cudaMemcpy(s->w, set, n * 4, cudaMemcpyHostToDevice));
    GAPGB_CUDA_TRY(cudaMemcpy(s->w16, w16.data(), n * 2, cudaMemcpyHostToDevice));
    GAPGB_CUDA_TRY(cudaMemset(s->m, 0, n * 4));
    GAPGB_CUDA_TRY(cudaMemset(s->v, 0, n * 4));
    s->step = 0;
  }
  return GAPGB_OK;
}

gapgb_status gapgb_surrogate_train_step(gapgb_surrogate *s, int rows_per_species, const int *d_rows,
                                        const float *d_G, const double *d_e, const float *d_dedg,
                                        float lambda, float lr, int update, double *loss,
                                        float *d_grad) {
  if (!s || !d_rows || !d_G || !d_e || !d_dedg) return sfail(GAPGB_ERR_ARG, "null argument");
  const int R = rows_per_species;
  if (R <= 0 || R % kTile) return sfail(GAPGB_ERR_ARG, "rows_per_species must be a positive multiple of 64");
  GAPGB_CUDA_TRY(cudaSetDevice(s->device));
  const int D = s->D, H = s->H, Q = s->members, nsp = s->nsp;
  const int rows = nsp * R;                 // rows per member
  const size_t total = (size_t)rows * Q;    // rows over all members
  gapgb_status st = ensure_rows(s, total);
  if (st) return st;
  if (R != s->train_R) {
    if (s->t_tile_sp) cudaFree(s->t_tile_sp);
    s->t_tile_sp = nullptr;
    s->train_R = 0;
    std::vector<int> ts(rows / kTile);
    for (size_t t = 0; t < ts.size(); ++t) ts[t] = (int)(t * kTile / R);
    if (!dalloc(&s->t_tile_sp, ts.size())) return sfail(GAPGB_ERR_ALLOC, "surrogate tile table");
    GAPGB_CUDA_TRY(cudaMemcpy(s->t_tile_sp, ts.data(), ts.size() * 4, cudaMemcpyHostToDevice));
    s->train_R = R;
  }
  cudaStream_t cs = s->stream;
  const size_t zH = (size_t)rows * H, zD = (size_t)rows * D;
  const int J = Q * nsp;  // (member, species) segments of R rows
  const size_t sH = (size_t)R * H, sD = (size_t)R * D;
  GAPGB_CUDA_TRY(cudaMemcpyAsync(s->idx, d_rows, total * sizeof(int), cudaMemcpyDeviceToDevice, cs));
  k_mlp_gather<<<nblk(total * D), 256, 0, cs>>>(total, D, s->idx, d_G, s->mu, s->isig, s->X);
  // tensor-core GEMMs when every 128-row tile lies in one species segment;
  // split-K scratch for the weight gradients (J blocks x up to 16 splits)
  int *tcf = (R % 128 == 0) ? s->t_err : nullptr;
  const size_t part_n = (size_t)Q * nsp * 16 * H * std::max(H, D);
  if (tcf && s->t_part_n < part_n) {
    if (s->t_part) cudaFree(s->t_part);
    s->t_part = nullptr;
    s->t_part_n = 0;
    if (dalloc(&s->t_part, part_n)) s->t_part_n = part_n;
    else cudaGetLastError();  // no scratch: the GEMMs run without splitting K
  }
  forward(s, cs, rows, s->t_tile_sp, zD, true, tcf);
  LossArgs la{R, nsp, D, lambda, 1.f / s->e_scale, s->idx, s->y, s->Gx, d_e, d_dedg, s->sd,
              s->e_shift, s->eps, s->Rv, s->R16, s->lrows};
  k_mlp_loss<<<nblk(total * 32), 256, 0, cs>>>(la, total);
  const size_t mstride = (size_t)nsp * s->P;
  const int *ts = s->t_tile_sp;
  // tangent pass along r
  gemm(cs, Q, rows, H, D, s->R16, D, 1, zD, s->w16 + s->W1, D, 1, mstride, ts, s->P, s->U1, H, zH, 0.f,
       tcf);
  k_mlp_dsilu<<<nblk(total * H), 256, 0, cs>>>(total * H, s->Z1, s->U1, nullptr, s->V1);
  gemm(cs, Q, rows, H, H, s->V1, H, 1, zH, s->w16 + s->W2, H, 1, mstride, ts, s->P, s->U2, H, zH, 0.f,
       tcf);
  // reverse pass, layer 2
  RowMap rm{rows, nsp, s->P, ts};
  k_mlp_back2<<<nblk(total * H), 256, 0, cs>>>(rm, Q, H, s->w3, s->w, s->Z2, s->U2, s->eps, s->Zb2, s->Ub2);
  k_mlp_grad_w3<<<dim3(nblk(H), J), 256, 0, cs>>>(R, H, s->P, s->w3, s->b3, s->Z2, s->U2, s->eps, s->grad);
  // dW2 = zbar2^T a1 + ubar2^T v1 per segment (M = N = H, K = R)
  gemm(cs, J, H, H, R, s->Zb2, 1, H, sH, s->A1, 1, H, sH, nullptr, 0, s->grad + s->W2, H, s->P, 0.f,
       tcf, s->t_part, s->t_part_n);
  gemm(cs, J, H, H, R, s->Ub2, 1, H, sH, s->V1, 1, H, sH, nullptr, 0, s->grad + s->W2, H, s->P, 1.f,
       tcf, s->t_part, s->t_part_n);
  k_mlp_colsum<<<dim3(nblk(H), J), 256, 0, cs>>>(R, H, s->P, s->b2, s->Zb2, s->grad);
  // abar1 = W2^T zbar2, vbar1 = W2^T ubar2
  gemm(cs, Q, rows, H, H, s->Zb2, H, 1, zH, s->w16 + s->W2, 1, H, mstride, ts, s->P, s->Ab1, H, zH, 0.f,
       tcf);
  gemm(cs, Q, rows, H, H, s->Ub2, H, 1, zH, s->w16 + s->W2, 1, H, mstride, ts, s->P, s->Vb1, H, zH, 0.f,
       tcf);
  k_mlp_back1<<<nblk(total * H), 256, 0, cs>>>(total * H, s->Z1, s->U1, s->Ab1, s->Vb1, s->Zb1, s->Ub1);
  // dW1 = zbar1^T x + ubar1^T r per segment (M = H, N = D, K = R)
  gemm(cs, J, H, D, R, s->Zb1, 1, H, sH, s->X, 1, D, sD, nullptr, 0, s->grad + s->W1, D, s->P, 0.f,
       tcf, s->t_part, s->t_part_n);
  gemm(cs, J, H, D, R, s->Ub1, 1, H, sH, s->R16, 1, D, sD, nullptr, 0, s->grad + s->W1, D, s->P, 1.f,
       tcf, s->t_part, s->t_part_n);
  k_mlp_colsum<<<dim3(nblk(H), J), 256, 0, cs>>>(R, H, s->P, s->b1, s->Zb1, s->grad);
  const size_t n = (size_t)J * s->P;
  if (d_grad) GAPGB_CUDA_TRY(cudaMemcpyAsync(d_grad, s->grad, n * 4, cudaMemcpyDeviceToDevice, cs));
  if (update) {
    s->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)s->step), c2 = 1.f - std::pow(b2, (float)s->step);
    k_mlp_adam<<<nblk(n), 256, 0, cs>>>(n, s->w, s->w16, s->m, s->v, s->grad, lr, b1, b2, 1e-8f, c1, c2);
  }
  GAPGB_CUDA_TRY(cudaGetLastError());
  if (loss) {
    std::vector<double> lr_h(total);
    int terr = 0;
    GAPGB_CUDA_TRY(cudaMemcpyAsync(lr_h.data(), s->lrows, total * sizeof(double), cudaMemcpyDeviceToHost, cs));
    GAPGB_CUDA_TRY(cudaMemcpyAsync(&terr, s->t_err, sizeof(int), cudaMemcpyDeviceToHost, cs));
    GAPGB_CUDA_TRY(cudaStreamSynchronize(cs));
    if (terr & kFlagTimeout) {
      cudaMemsetAsync(s->t_err, 0, sizeof(int), cs);
      return sfail(GAPGB_ERR_TIMEOUT, "a bounded tensor-core wait of the training GEMMs gave up");
    }
    for (int z = 0; z < J; ++z)
      loss[z] = std::accumulate(lr_h.begin() + (size_t)z * R, lr_h.begin() + (size_t)(z + 1) * R, 0.0) / R;
  }
  return GAPGB_OK;
}

gapgb_status gapgb_surrogate_predict(gapgb_surrogate *s, int natoms, const int *d_species,
                                     const float *d_G, double *d_e, float *d_std, float *d_dedg,
                                     float *d_gstd, void *stream) {
  if (!s || !d_species || !d_G || !d_e || !d_std || !d_dedg) return sfail(GAPGB_ERR_ARG, "null argument");
  if (natoms <= 0) return sfail(GAPGB_ERR_ARG, "natoms must be positive");
  GAPGB_CUDA_TRY(cudaSetDevice(s->device));
  gapgb_status st = surrogate_prepare(s, natoms);
  if (st) return st;
  cudaStream_t cs = stream ? (cudaStream_t)stream : s->stream;
  GAPGB_CUDA_TRY(cudaMemsetAsync(s->p_err, 0, sizeof(int), cs));
  surrogate_enqueue(s, natoms, d_species, d_G, d_e, d_std, d_dedg, d_gstd, s->p_err, cs);
  GAPGB_CUDA_TRY(cudaGetLastError());
  int err = 0;
  GAPGB_CUDA_TRY(cudaMemcpyAsync(&err, s->p_err, sizeof(int), cudaMemcpyDeviceToHost, cs));
  GAPGB_CUDA_TRY(cudaStreamSynchronize(cs));
  if (err & kFlagUnknownSpecies)
    return sfail(GAPGB_ERR_UNKNOWN_SPECIES, "atomic number absent from the surrogate's species");
  return GAPGB_OK;
}

}  // extern "C"
