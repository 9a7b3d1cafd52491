// wacsf.cu - weighted atom-centred symmetry functions and their gradients.
//
// Reference: CAR2ACSF, gappy/libgap/wacsf.f90:58-795.
//   type 1  G = sum_j exp(-alpha r_ij^2) fc(r_ij)                  (:69-162)
//   type 3  G = sum_j exp(-4 (r_ij - R_s)^2) fc(r_ij)              (:436-527)
//   type 2  G = sum_{j<k} (1 + cos) exp(-alpha (rij^2+rik^2+rjk^2)) fc fc fc   (:169-432)
//   type 4  as type 2 with (1 - cos)                               (:534-791)
//   fc(r) = 0.5 (cos(pi r / rc) + 1) with pi = 3.141592654, terms kept
//   when r <= rc (the reference skips r > rc); descriptor d holds the
//   unweighted sum and d + nsf the sum weighted by w_j (radial) or w_j w_k
//   (angular) (:86-87, :326-328).  Optional extension: angular zeta, with
//   2^(1-zeta) (1 +- cos)^zeta; zeta = 1 is the reference.
//
// The reference stores the dense Jacobian dxdy(D,N,N,3) and strs(3,3,D,N)
// and contracts it with dE/dG afterwards (gap_calc.f90:177-200).  Here the
// gradient pass runs after the GPR and contracts on the fly: for atom i and
// neighbour slot q (an image position p_q) it writes
//     gslot[i][q] = sum_d dE/dG_id * dG_id/dp_q
// and the per-atom virial sum_q (p_q - r_i) (x) gslot[i][q]; forces follow by
// a gather over reverse slots (reduce.cu).  No N x N array exists.
//
// Work layout: one warp per centre atom.  The warp stages its neighbour
// slots (relative vectors, distances, weights) and per-slot tables
// fc(r_q), fc'(r_q) for every distinct cutoff and exp(-alpha r_q^2) for every
// distinct angular alpha in shared memory.  Forward: lanes take slots
// (radial) and pairs of the upper triangle (angular) and accumulate into a
// per-lane column of a shared [D][32] array, summed in lane order at the end.
// Backward: radial terms by slot (each lane owns its slots); angular pairs in
// the rounds of a round-robin tournament schedule, in which every slot
// appears in at most one pair per round, so lanes update slot gradients in
// shared memory without atomics and the result is deterministic.
#include "gapgb_internal.h"

namespace gapgb {
namespace {

__device__ __forceinline__ double t_exp(double x) { return exp(x); }
__device__ __forceinline__ float t_exp(float x) { return expf(x); }
__device__ __forceinline__ double t_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float t_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double t_cos(double x) { return cos(x); }
__device__ __forceinline__ float t_cos(float x) { return cosf(x); }
__device__ __forceinline__ void t_sincos(double x, double *s, double *c) { sincos(x, s, c); }
__device__ __forceinline__ void t_sincos(float x, float *s, float *c) { sincosf(x, s, c); }
__device__ __forceinline__ double t_pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float t_pow(float x, float y) { return powf(x, y); }

// pref * base^zeta and its derivative with respect to base.
template <typename T>
__device__ __forceinline__ void ang_factor(T base, int iz, T zeta, T pref, T *A, T *dA) {
  if (iz == 1) {
    *A = base;
    *dA = (T)1;
  } else if (iz > 1) {
    T p = base;
    for (int t = 2; t < iz; ++t) p *= base;  // base^(iz-1)
    *dA = pref * (T)iz * p;
    *A = pref * p * base;
  } else {
    T b = base > (T)0 ? base : (T)0;
    T p = t_pow(b, zeta - (T)1);
    *dA = pref * zeta * p;
    *A = pref * p * b;
  }
}

template <typename T>
struct Layout {
  T *dx, *dy, *dz, *r, *w, *fc, *dfc, *ea, *ec, *acc, *gx, *gy, *gz, *dg;
};

template <typename T>
__device__ __forceinline__ Layout<T> carve(unsigned char *raw, int warp, int capS, int nrc, int nal,
                                           int D, bool fwd) {
  const size_t per = (size_t)5 * capS + (size_t)nrc * capS * (fwd ? 1 : 2) + (size_t)nal * capS +
                     (size_t)nal * 32 + (fwd ? (size_t)D * 32 : (size_t)3 * capS + D);
  T *b = reinterpret_cast<T *>(raw) + per * warp;
  Layout<T> L;
  L.dx = b;
  L.dy = L.dx + capS;
  L.dz = L.dy + capS;
  L.r = L.dz + capS;
  L.w = L.r + capS;
  L.fc = L.w + capS;
  L.dfc = L.fc + (size_t)nrc * capS;
  L.ea = fwd ? L.dfc : L.dfc + (size_t)nrc * capS;
  L.ec = L.ea + (size_t)nal * capS;
  T *rest = L.ec + (size_t)nal * 32;
  if (fwd) {
    L.acc = rest;
    L.gx = L.gy = L.gz = L.dg = nullptr;
  } else {
    L.acc = nullptr;
    L.gx = rest;
    L.gy = L.gx + capS;
    L.gz = L.gy + capS;
    L.dg = L.gz + capS;
  }
  return L;
}

// Stage the slots of atom i and the per-slot cutoff / exponential tables.
template <typename T>
__device__ __forceinline__ int stage_slots(const Layout<T> &L, int i, int cap, int capS, int lane,
                                           const int *__restrict__ cnt,
                                           const double4 *__restrict__ xyzr,
                                           const int *__restrict__ nj,
                                           const double4 *__restrict__ apos,
                                           const SFDev *__restrict__ sf, bool want_dfc) {
  const int P = min(cnt[i], capS);
  const double4 pi = apos[i];
  const T PI = (T)kPiRef;
  const int nrc = sf->nrc, nal = sf->nalpha;
  for (int q = lane; q < P; q += 32) {
    const double4 e = xyzr[(size_t)i * cap + q];
    const int j = nj[(size_t)i * cap + q];
    // deltaxj = -(pos(i) - xyz) (wacsf.f90:90)
    L.dx[q] = (T)(e.x - pi.x);
    L.dy[q] = (T)(e.y - pi.y);
    L.dz[q] = (T)(e.z - pi.z);
    const T r = (T)e.w;
    L.r[q] = r;
    L.w[q] = (T)apos[j].w;
    for (int g = 0; g < nrc; ++g) {
      const T rc = (T)sf->rc_val[g];
      T fcv = (T)0, dfcv = (T)0;
      if (r <= rc) {
        const T x = PI * r / rc;
        if (want_dfc) {
          T sn, cs;
          t_sincos(x, &sn, &cs);
          fcv = (T)0.5 * (cs + (T)1);
          dfcv = (T)0.5 * (-sn) * (PI / rc);
        } else {
          fcv = (T)0.5 * (t_cos(x) + (T)1);
        }
      }
      L.fc[(size_t)g * capS + q] = fcv;
      if (want_dfc) L.dfc[(size_t)g * capS + q] = dfcv;
    }
    for (int a = 0; a < nal; ++a) L.ea[(size_t)a * capS + q] = t_exp(-(T)sf->alpha_val[a] * r * r);
  }
  return P;
}

template <typename T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    k_wacsf_fwd(int N, int cap, int capS, const int *__restrict__ cnt,
                const double4 *__restrict__ xyzr, const int *__restrict__ nj,
                const double4 *__restrict__ apos, const SFDev *__restrict__ sf,
                T *__restrict__ G) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nrc = sf->nrc, nal = sf->nalpha, D = sf->D, nsf = sf->nsf;
  const int nrad = sf->nrad, ngrp = sf->n_ang_grp;
  const Layout<T> L = carve<T>(smraw, warp, capS, nrc, nal, D, true);
  const T PI = (T)kPiRef;
  const T maxrc = (T)sf->max_ang_rc;
  for (int i = blockIdx.x * kWarpsPerBlock + warp; i < N; i += gridDim.x * kWarpsPerBlock) {
    const int P = stage_slots<T>(L, i, cap, capS, lane, cnt, xyzr, nj, apos, sf, false);
    for (int d = 0; d < D; ++d) L.acc[d * 32 + lane] = (T)0;
    __syncwarp();
    // radial terms: lanes own slots
    for (int q = lane; q < P; q += 32) {
      const T r = L.r[q], w = L.w[q];
      for (int s = 0; s < nrad; ++s) {
        const T f = L.fc[(size_t)sf->rad_rc[s] * capS + q];
        if (r > (T)sf->rc_val[sf->rad_rc[s]]) continue;
        const T u = r - (T)sf->rad_rs[s];
        const T v = t_exp(-(T)sf->rad_alpha[s] * u * u) * f;
        const int d = sf->rad_d[s];
        L.acc[d * 32 + lane] += v;
        L.acc[(d + nsf) * 32 + lane] += v * w;
      }
    }
    // angular terms: lanes walk the upper triangle j < k with stride 32
    if (sf->nang > 0 && P > 1) {
      const int npair = P * (P - 1) / 2;
      int j = 0, k = 1 + lane;
      while (j < P - 1 && k >= P) { const int o = k - P; ++j; k = j + 1 + o; }
      for (int p = lane; p < npair; p += 32) {
        const T a = L.r[j], b = L.r[k];
        if (a <= maxrc && b <= maxrc) {
          const T cx = L.dx[j] - L.dx[k], cy = L.dy[j] - L.dy[k], cz = L.dz[j] - L.dz[k];
          const T c2 = cx * cx + cy * cy + cz * cz;
          const T c = t_sqrt(c2);
          if (c <= maxrc) {
            // costheta = f/g, f = rjk^2 - rij^2 - rik^2, g = -2 rij rik (wacsf.f90:271-273)
            const T cosv = (c2 - a * a - b * b) / ((T)-2 * a * b);
            for (int al = 0; al < nal; ++al) L.ec[al * 32 + lane] = t_exp(-(T)sf->alpha_val[al] * c2);
            const T wjk = L.w[j] * L.w[k];
            for (int g = 0; g < ngrp; ++g) {
              const int rci = sf->ang_grp_rc[g];
              const T rc = (T)sf->rc_val[rci];
              if (a > rc || b > rc || c > rc) continue;
              const T F = L.fc[(size_t)rci * capS + j] * L.fc[(size_t)rci * capS + k] *
                          ((T)0.5 * (t_cos(PI * c / rc) + (T)1));
              for (int s = sf->ang_grp_start[g]; s < sf->ang_grp_start[g + 1]; ++s) {
                const int al = sf->ang_alpha[s];
                T A, dA;
                ang_factor<T>((T)1 + (T)sf->ang_lambda[s] * cosv, sf->ang_izeta[s],
                              (T)sf->ang_zeta[s], (T)sf->ang_pref[s], &A, &dA);
                const T E = L.ea[(size_t)al * capS + j] * L.ea[(size_t)al * capS + k] *
                            L.ec[al * 32 + lane];
                const T v = A * E * F;
                const int d = sf->ang_d[s];
                L.acc[d * 32 + lane] += v;
                L.acc[(d + nsf) * 32 + lane] += v * wjk;
              }
            }
          }
        }
        k += 32;
        while (j < P - 1 && k >= P) { const int o = k - P; ++j; k = j + 1 + o; }
      }
    }
    __syncwarp();
    for (int d = lane; d < D; d += 32) {
      T s = (T)0;
      for (int l = 0; l < 32; ++l) s += L.acc[d * 32 + l];
      G[(size_t)i * D + d] = s;
    }
    __syncwarp();
  }
}

template <typename T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    k_wacsf_bwd(int N, int cap, int capS, const int *__restrict__ cnt,
                const double4 *__restrict__ xyzr, const int *__restrict__ nj,
                const double4 *__restrict__ apos, const SFDev *__restrict__ sf,
                const T *__restrict__ dedg, typename Vec4<T>::type *__restrict__ gslot,
                double *__restrict__ wvir) {
  using V4 = typename Vec4<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nrc = sf->nrc, nal = sf->nalpha, D = sf->D, nsf = sf->nsf;
  const int nrad = sf->nrad, ngrp = sf->n_ang_grp;
  const Layout<T> L = carve<T>(smraw, warp, capS, nrc, nal, D, false);
  const T PI = (T)kPiRef;
  const T maxrc = (T)sf->max_ang_rc;
  for (int i = blockIdx.x * kWarpsPerBlock + warp; i < N; i += gridDim.x * kWarpsPerBlock) {
    const int P = stage_slots<T>(L, i, cap, capS, lane, cnt, xyzr, nj, apos, sf, true);
    for (int d = lane; d < D; d += 32) L.dg[d] = dedg[(size_t)i * D + d];
    for (int q = lane; q < P; q += 32) L.gx[q] = L.gy[q] = L.gz[q] = (T)0;
    __syncwarp();
    // radial terms
    for (int q = lane; q < P; q += 32) {
      const T r = L.r[q], w = L.w[q];
      T S = (T)0;
      for (int s = 0; s < nrad; ++s) {
        const int rci = sf->rad_rc[s];
        if (r > (T)sf->rc_val[rci]) continue;
        const T f = L.fc[(size_t)rci * capS + q], df = L.dfc[(size_t)rci * capS + q];
        const T alpha = (T)sf->rad_alpha[s];
        const T u = r - (T)sf->rad_rs[s];
        const T ex = t_exp(-alpha * u * u);
        const T dphi = (T)-2 * alpha * u * ex * f + ex * df;
        const int d = sf->rad_d[s];
        S += (L.dg[d] + L.dg[d + nsf] * w) * dphi;
      }
      const T ir = (T)1 / r;
      L.gx[q] += S * L.dx[q] * ir;
      L.gy[q] += S * L.dy[q] * ir;
      L.gz[q] += S * L.dz[q] * ir;
    }
    __syncwarp();
    // angular terms in round-robin rounds (circle method over Pp slots)
    if (sf->nang > 0 && P > 1) {
      const int Pp = P + (P & 1);
      const int half = Pp >> 1;
      for (int round = 0; round < Pp - 1; ++round) {
        for (int t = lane; t < half; t += 32) {
          int j, k;
          if (t == 0) {
            j = Pp - 1;
            k = round;
          } else {
            j = (round + t) % (Pp - 1);
            k = (round - t + Pp - 1) % (Pp - 1);
          }
          if (j >= P || k >= P) continue;
          const T a = L.r[j], b = L.r[k];
          if (a > maxrc || b > maxrc) continue;
          const T djx = L.dx[j], djy = L.dy[j], djz = L.dz[j];
          const T dkx = L.dx[k], dky = L.dy[k], dkz = L.dz[k];
          const T cx = djx - dkx, cy = djy - dky, cz = djz - dkz;
          const T c2 = cx * cx + cy * cy + cz * cz;
          const T c = t_sqrt(c2);
          if (c > maxrc) continue;
          const T cosv = (c2 - a * a - b * b) / ((T)-2 * a * b);
          const T ia = (T)1 / a, ib = (T)1 / b, ic = (T)1 / c;
          const T dcda = ib - cosv * ia;  // d cos / d r_ij
          const T dcdb = ia - cosv * ib;  // d cos / d r_ik
          const T dcdc = -c * ia * ib;    // d cos / d r_jk
          for (int al = 0; al < nal; ++al) L.ec[al * 32 + lane] = t_exp(-(T)sf->alpha_val[al] * c2);
          const T wjk = L.w[j] * L.w[k];
          T S1 = (T)0, S2 = (T)0, S3 = (T)0;
          for (int g = 0; g < ngrp; ++g) {
            const int rci = sf->ang_grp_rc[g];
            const T rc = (T)sf->rc_val[rci];
            if (a > rc || b > rc || c > rc) continue;
            const T fa = L.fc[(size_t)rci * capS + j], fb = L.fc[(size_t)rci * capS + k];
            const T dfa = L.dfc[(size_t)rci * capS + j], dfb = L.dfc[(size_t)rci * capS + k];
            T sn, cs;
            t_sincos(PI * c / rc, &sn, &cs);
            const T fcc = (T)0.5 * (cs + (T)1);
            const T dfcc = (T)0.5 * (-sn) * (PI / rc);
            const T F = fa * fb * fcc;
            for (int s = sf->ang_grp_start[g]; s < sf->ang_grp_start[g + 1]; ++s) {
              const int al = sf->ang_alpha[s];
              const T lam = (T)sf->ang_lambda[s];
              T A, dA;
              ang_factor<T>((T)1 + lam * cosv, sf->ang_izeta[s], (T)sf->ang_zeta[s],
                            (T)sf->ang_pref[s], &A, &dA);
              const T Ap = dA * lam;  // d A / d cos
              const T E = L.ea[(size_t)al * capS + j] * L.ea[(size_t)al * capS + k] *
                          L.ec[al * 32 + lane];
              const T alpha = (T)sf->alpha_val[al];
              const T AE = A * E;
              const T EF = E * F;
              const T m2a = (T)-2 * alpha * AE * F;
              const int d = sf->ang_d[s];
              const T cs_ = L.dg[d] + L.dg[d + nsf] * wjk;
              S1 += cs_ * (Ap * dcda * EF + m2a * a + AE * dfa * fb * fcc);
              S2 += cs_ * (Ap * dcdb * EF + m2a * b + AE * fa * dfb * fcc);
              S3 += cs_ * (Ap * dcdc * EF + m2a * c + AE * fa * fb * dfcc);
            }
          }
          const T s1 = S1 * ia, s2 = S2 * ib, s3 = S3 * ic;
          L.gx[j] += s1 * djx + s3 * cx;
          L.gy[j] += s1 * djy + s3 * cy;
          L.gz[j] += s1 * djz + s3 * cz;
          L.gx[k] += s2 * dkx - s3 * cx;
          L.gy[k] += s2 * dky - s3 * cy;
          L.gz[k] += s2 * dkz - s3 * cz;
        }
        __syncwarp();
      }
    }
    __syncwarp();
    // write slot gradients and the per-atom virial (FP64 accumulation)
    double W[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = lane; q < P; q += 32) {
      const T gx = L.gx[q], gy = L.gy[q], gz = L.gz[q];
      V4 v;
      v.x = gx;
      v.y = gy;
      v.z = gz;
      v.w = (T)0;
      gslot[(size_t)i * cap + q] = v;
      const double d3[3] = {(double)L.dx[q], (double)L.dy[q], (double)L.dz[q]};
      const double g3[3] = {(double)gx, (double)gy, (double)gz};
#pragma unroll
      for (int aa = 0; aa < 3; ++aa)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) W[aa * 3 + bb] += d3[aa] * g3[bb];
    }
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      double v = W[t];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      W[t] = v;
    }
    if (lane < 9) wvir[(size_t)i * 9 + lane] = W[lane];
    __syncwarp();
  }
}

int warp_grid(int N, size_t smem_per_block, const void *fn) {
  int dev = 0, sms = 148, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * kWarpsPerBlock, smem_per_block);
  if (per_sm < 1) per_sm = 1;
  int need = (N + kWarpsPerBlock - 1) / kWarpsPerBlock;
  int maxb = sms * per_sm;
  return need < maxb ? (need > 0 ? need : 1) : maxb;
}

}  // namespace

size_t wacsf_smem_bytes(const SFDev &t, int capS, bool fwd, size_t elem) {
  const size_t per = (size_t)5 * capS + (size_t)t.nrc * capS * (fwd ? 1 : 2) +
                     (size_t)t.nalpha * capS + (size_t)t.nalpha * 32 +
                     (fwd ? (size_t)t.D * 32 : (size_t)3 * capS + t.D);
  return per * elem * kWarpsPerBlock;
}

template <typename T>
void launch_wacsf_fwd(const gapgb_model *m, Workspace &ws, int N, int cap, int capS,
                      cudaStream_t st) {
  const size_t smem = wacsf_smem_bytes(m->sfh, capS, true, sizeof(T));
  auto fn = k_wacsf_fwd<T>;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int grid = warp_grid(N, smem, (const void *)fn);
  fn<<<grid, 32 * kWarpsPerBlock, smem, st>>>(N, cap, capS, ws.nbr_cnt, ws.nbr_xyz, ws.nbr_j,
                                               ws.apos, m->d_sf, (T *)ws.G);
}

template <typename T>
void launch_wacsf_bwd(const gapgb_model *m, Workspace &ws, int N, int cap, int capS,
                      cudaStream_t st) {
  const size_t smem = wacsf_smem_bytes(m->sfh, capS, false, sizeof(T));
  auto fn = k_wacsf_bwd<T>;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int grid = warp_grid(N, smem, (const void *)fn);
  fn<<<grid, 32 * kWarpsPerBlock, smem, st>>>(N, cap, capS, ws.nbr_cnt, ws.nbr_xyz, ws.nbr_j,
                                               ws.apos, m->d_sf, (const T *)ws.dedg,
                                               (typename Vec4<T>::type *)ws.gslot, ws.wvir);
}

template void launch_wacsf_fwd<double>(const gapgb_model *, Workspace &, int, int, int, cudaStream_t);
template void launch_wacsf_fwd<float>(const gapgb_model *, Workspace &, int, int, int, cudaStream_t);
template void launch_wacsf_bwd<double>(const gapgb_model *, Workspace &, int, int, int, cudaStream_t);
template void launch_wacsf_bwd<float>(const gapgb_model *, Workspace &, int, int, int, cudaStream_t);

}  // namespace gapgb
