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
// a gather over reverse slots (reduce.cu), or, in the grouped FP32 kernels
// (wacsf_grouped.cuh), by a scatter in the gradient kernel itself.  No N x N
// array exists.
//
// Work layout: one warp per centre atom.  The warp stages its neighbour
// slots (relative vectors, distances, weights) and per-slot tables
// fc(r_q), fc'(r_q) (zero beyond each cutoff, so a term outside a cutoff
// contributes exactly zero) and exp(-alpha r_q^2) in shared memory; the block
// stages the SF table in the kernel's arithmetic type.
// Forward: radial SFs one per lane over the slots in order (registers);
// angular SFs in chunks of 16 register accumulators per lane over the pairs
// of the upper triangle, summed over lanes by a fixed shuffle tree.
// Backward: radial terms by slot (each lane owns its slots); angular pairs in
// the rounds of a round-robin tournament schedule, in which every slot
// appears in at most one pair per round, so lanes update slot gradients in
// shared memory without atomics and the result is deterministic.
#include <type_traits>

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

// Non-integer zeta (rare): kept out of line so that the unrolled SF loops
// stay small.
template <typename T>
__device__ __noinline__ T pow_general(T base, T zeta, T *dA) {
  const T b = base > (T)0 ? base : (T)0;
  const T p = t_pow(b, zeta - (T)1);
  *dA = zeta * p;
  return p * b;
}

// base^zeta and its derivative with respect to base (2^(1-zeta) applied by
// the caller); iz = integer zeta, 0 for a non-integer zeta.
template <typename T>
__device__ __forceinline__ void ang_pow(T base, int iz, T zeta, T *A, T *dA) {
  if (iz == 1) {
    *A = base;
    *dA = (T)1;
  } else if (iz > 1) {
    T p = base;
    for (int t = 2; t < iz; ++t) p *= base;  // base^(iz-1)
    *dA = (T)iz * p;
    *A = p * base;
  } else {
    *A = pow_general<T>(base, zeta, dA);
  }
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

__host__ __device__ constexpr size_t kTableBytes(size_t s) { return (s + 15) / 16 * 16; }

template <typename T>
struct Layout {
  T *dx, *dy, *dz, *r, *w, *ir, *fc, *dfc, *ea, *Fp, *Ep, *gx, *gy, *gz, *dg, *cA, *cB;
};

template <typename T>
__host__ __device__ __forceinline__ size_t per_warp_elems(int capS, int nrc, int nal, int D,
                                                          int nang, bool fwd) {
  return fwd ? (size_t)6 * capS + (size_t)nrc * capS + (size_t)nal * capS + (size_t)nrc * 32 +
                   (size_t)nal * 32
             : (size_t)6 * capS + (size_t)2 * nrc * capS + (size_t)nal * capS +
                   (size_t)nal * 32 + (size_t)3 * capS + D + (size_t)2 * nang;
}

template <typename T>
__device__ __forceinline__ Layout<T> carve(unsigned char *raw, int warp, int capS, int nrc,
                                           int nal, int D, int nang, bool fwd) {
  T *b = reinterpret_cast<T *>(raw + kTableBytes(sizeof(SFT<T>))) +
         per_warp_elems<T>(capS, nrc, nal, D, nang, fwd) * warp;
  Layout<T> L;
  L.dx = b;
  L.dy = L.dx + capS;
  L.dz = L.dy + capS;
  L.r = L.dz + capS;
  L.w = L.r + capS;
  L.ir = L.w + capS;
  L.fc = L.ir + capS;
  L.dfc = L.fc + (size_t)nrc * capS;
  L.ea = fwd ? L.dfc : L.dfc + (size_t)nrc * capS;
  T *p = L.ea + (size_t)nal * capS;
  if (fwd) {
    L.Fp = p;
    L.Ep = L.Fp + (size_t)nrc * 32;
    L.gx = L.gy = L.gz = L.dg = L.cA = L.cB = nullptr;
  } else {
    L.Fp = nullptr;
    L.Ep = p;
    L.gx = L.Ep + (size_t)nal * 32;
    L.gy = L.gx + capS;
    L.gz = L.gy + capS;
    L.dg = L.gz + capS;
    L.cA = L.dg + D;
    L.cB = L.cA + nang;
  }
  return L;
}

template <typename T>
__device__ __forceinline__ void load_table(unsigned char *raw, const SFT<T> *__restrict__ g) {
  const int n = (int)(sizeof(SFT<T>) / 4);
  for (int q = threadIdx.x; q < n; q += blockDim.x)
    reinterpret_cast<int *>(raw)[q] = reinterpret_cast<const int *>(g)[q];
  __syncthreads();
}

// Slot geometry: FP64 from the image positions, FP32 from the FP32 records
// the neighbour kernel wrote (one rounding of the FP64 difference).
__device__ __forceinline__ void slot_geom(int i, int q, int cap, const double4 &pi,
                                          const double4 *__restrict__ xyzr,
                                          const int *__restrict__ nj,
                                          const double4 *__restrict__ apos,
                                          const float4 *__restrict__ d32,
                                          const float *__restrict__ w32, double *dx, double *dy,
                                          double *dz, double *r, double *w) {
  (void)d32;
  (void)w32;
  const double4 e = xyzr[(size_t)i * cap + q];
  *dx = e.x - pi.x;  // deltaxj = -(pos(i) - xyz) (wacsf.f90:90)
  *dy = e.y - pi.y;
  *dz = e.z - pi.z;
  *r = e.w;
  *w = apos[nj[(size_t)i * cap + q]].w;
}
__device__ __forceinline__ void slot_geom(int i, int q, int cap, const double4 &pi,
                                          const double4 *__restrict__ xyzr,
                                          const int *__restrict__ nj,
                                          const double4 *__restrict__ apos,
                                          const float4 *__restrict__ d32,
                                          const float *__restrict__ w32, float *dx, float *dy,
                                          float *dz, float *r, float *w) {
  (void)pi;
  (void)xyzr;
  (void)nj;
  (void)apos;
  const float4 e = d32[(size_t)i * cap + q];
  *dx = e.x;
  *dy = e.y;
  *dz = e.z;
  *r = e.w;
  *w = w32[(size_t)i * cap + q];
}

template <typename T>
__device__ __forceinline__ int stage_slots(const Layout<T> &L, const SFT<T> &sf, int i, int cap,
                                           int capS, int lane, const int *__restrict__ cnt,
                                           const double4 *__restrict__ xyzr,
                                           const int *__restrict__ nj,
                                           const double4 *__restrict__ apos,
                                           const float4 *__restrict__ d32,
                                           const float *__restrict__ w32, bool want_dfc) {
  const int P = min(cnt[i], capS);
  double4 pi = make_double4(0, 0, 0, 0);
  if (sizeof(T) == 8) pi = apos[i];
  const int nrc = sf.nrc, nal = sf.nalpha;
  for (int q = lane; q < P; q += 32) {
    T dx, dy, dz, r, w;
    slot_geom(i, q, cap, pi, xyzr, nj, apos, d32, w32, &dx, &dy, &dz, &r, &w);
    L.dx[q] = dx;
    L.dy[q] = dy;
    L.dz[q] = dz;
    L.r[q] = r;
    L.w[q] = w;
    L.ir[q] = (T)1 / r;
    for (int g = 0; g < nrc; ++g) {
      T fcv = (T)0, dfcv = (T)0;
      if (r <= sf.rc_val[g]) {
        const T x = sf.pi_over_rc[g] * r;
        if (want_dfc) {
          T sn, cs;
          t_sincos(x, &sn, &cs);
          fcv = (T)0.5 * (cs + (T)1);
          dfcv = (T)-0.5 * sn * sf.pi_over_rc[g];
        } else {
          fcv = (T)0.5 * (t_cos(x) + (T)1);
        }
      }
      L.fc[(size_t)g * capS + q] = fcv;
      if (want_dfc) L.dfc[(size_t)g * capS + q] = dfcv;
    }
    for (int a = 0; a < nal; ++a) L.ea[(size_t)a * capS + q] = t_exp(-sf.alpha_val[a] * r * r);
  }
  return P;
}

// FP32: at least 4 blocks (16 warps) per SM; FP64 is FP64-pipe bound and
// keeps its registers.
// the parts an atom's pair (or round) loop is split into: a team of this
// many warps runs them side by side, a single warp in turn
constexpr int kTeam = kWarpsPerBlock;

// team = 1: one warp per atom.  team = kWarpsPerBlock (small batches, which
// would leave most SMs idle): the block's warps share one atom, each staging
// its own copy of the slots and taking every team-th 32-pair stride of the
// pair loop; their per-SF sums are added in warp order (deterministic).
template <typename T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, sizeof(T) == 4 ? 4 : 1)
    k_wacsf_fwd(int N, int cap, int capS, const int *__restrict__ cnt,
                const double4 *__restrict__ xyzr, const int *__restrict__ nj,
                const double4 *__restrict__ apos, const float4 *__restrict__ d32,
                const float *__restrict__ w32, const SFT<T> *__restrict__ sfg,
                T *__restrict__ G, int team) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ T s_part[kWarpsPerBlock][2 * kAngChunk];
  load_table<T>(smraw, sfg);
  const SFT<T> &sf = *reinterpret_cast<const SFT<T> *>(smraw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nrc = sf.nrc, nal = sf.nalpha, D = sf.D, nsf = sf.nsf;
  const int nrad = sf.nrad, nang = sf.nang, ngrp = sf.n_ang_grp;
  const Layout<T> L = carve<T>(smraw, warp, capS, nrc, nal, D, nang, true);
  const T maxrc = sf.max_ang_rc;
  const int tw = team > 1 ? warp : 0;  // this warp's place in its team
  const int per_block = team > 1 ? 1 : kWarpsPerBlock;
  for (int i = blockIdx.x * per_block + (team > 1 ? 0 : warp); i < N; i += gridDim.x * per_block) {
    const int P = stage_slots<T>(L, sf, i, cap, capS, lane, cnt, xyzr, nj, apos, d32, w32, false);
    __syncwarp();
    T *Gi = G + (size_t)i * D;
    // radial: one SF per lane, slots in the reference's order
    for (int s = lane + 32 * tw; s < nrad; s += 32 * team) {
      const int rci = sf.rad_rc[s];
      const T alpha = sf.rad_alpha[s], rs = sf.rad_rs[s];
      const T *fcr = L.fc + (size_t)rci * capS;
      T acc = (T)0, accw = (T)0;
      for (int q = 0; q < P; ++q) {
        const T f = fcr[q];
        if (f == (T)0) continue;  // beyond the cutoff (or exactly at it: a zero term)
        const T u = L.r[q] - rs;
        const T v = t_exp(-alpha * u * u) * f;
        acc += v;
        accw += v * L.w[q];
      }
      const int d = sf.rad_d[s];
      Gi[d] = acc;
      Gi[d + nsf] = accw;
    }
    // angular: chunks of kAngChunk SFs accumulated in registers.  The pairs
    // fall into kTeam parts (part w: the 32-pair strides w, w + kTeam, ...),
    // each summed on its own and the parts added in order into s_part,
    // whether one warp runs the parts in turn (team = 1) or the block's warps
    // run one part each: the rounding is the same for every launch shape, so
    // an atom's descriptors do not depend on the batch around it
    for (int c0 = 0; c0 < nang; c0 += kAngChunk) {
      int code[kAngChunk];
#pragma unroll
      for (int s = 0; s < kAngChunk; ++s) code[s] = (c0 + s < nang) ? sf.ang_code[c0 + s] : -1;
      if (lane < 2 * kAngChunk) s_part[warp][lane] = (T)0;
      __syncwarp();
      const int part0 = team > 1 ? tw : 0, part1 = team > 1 ? tw + 1 : kTeam;
      for (int part = part0; part < part1; ++part) {
        T accA[kAngChunk], accW[kAngChunk];
#pragma unroll
        for (int s = 0; s < kAngChunk; ++s) accA[s] = accW[s] = (T)0;
        if (P > 1) {
          const int npair = P * (P - 1) / 2;
          int j = 0, k = 1 + lane + 32 * part;
          while (j < P - 1 && k >= P) { const int o = k - P; ++j; k = j + 1 + o; }
          for (int p = lane + 32 * part; p < npair; p += 32 * kTeam) {
            const T a = L.r[j], b = L.r[k];
            if (a <= maxrc && b <= maxrc) {
              const T cx = L.dx[j] - L.dx[k], cy = L.dy[j] - L.dy[k], cz = L.dz[j] - L.dz[k];
              const T c2 = cx * cx + cy * cy + cz * cz;
              const T c = t_sqrt(c2);
              if (c <= maxrc) {
                // costheta = f/g, f = rjk^2 - rij^2 - rik^2, g = -2 rij rik (wacsf.f90:271-273)
                const T cosv = (c2 - a * a - b * b) / ((T)-2 * a * b);
                for (int g = 0; g < ngrp; ++g) {
                  const int rci = sf.ang_grp_rc[g];
                  const T fcc = (c <= sf.rc_val[rci])
                                    ? (T)0.5 * (t_cos(sf.pi_over_rc[rci] * c) + (T)1) : (T)0;
                  L.Fp[rci * 32 + lane] =
                      L.fc[(size_t)rci * capS + j] * L.fc[(size_t)rci * capS + k] * fcc;
                }
                for (int al = 0; al < nal; ++al)
                  L.Ep[al * 32 + lane] = L.ea[(size_t)al * capS + j] *
                                         L.ea[(size_t)al * capS + k] *
                                         t_exp(-sf.alpha_val[al] * c2);
                const T wjk = L.w[j] * L.w[k];
#pragma unroll
                for (int s = 0; s < kAngChunk; ++s) {
                  if (code[s] < 0) continue;
                  const int rci = code[s] & 255, al = (code[s] >> 8) & 255;
                  const int iz = (code[s] >> 16) & 255;
                  const T base = (code[s] >> 24) ? (T)1 - cosv : (T)1 + cosv;
                  T A, dA;
                  ang_pow<T>(base, iz, iz ? (T)1 : sf.ang_zeta[c0 + s], &A, &dA);
                  const T v = A * L.Ep[al * 32 + lane] * L.Fp[rci * 32 + lane];
                  accA[s] += v;
                  accW[s] += v * wjk;
                }
              }
            }
            k += 32 * kTeam;
            while (j < P - 1 && k >= P) { const int o = k - P; ++j; k = j + 1 + o; }
          }
        }
#pragma unroll
        for (int s = 0; s < kAngChunk; ++s) {
          const T x = warp_sum(accA[s]), y = warp_sum(accW[s]);
          if (lane == 0) {
            s_part[warp][s] += x;
            s_part[warp][kAngChunk + s] += y;
          }
        }
        __syncwarp();
      }
      if (team > 1) __syncthreads();
      if ((team > 1 ? warp == 0 : true) && lane < kAngChunk && c0 + lane < nang) {
        T x = (T)0, y = (T)0;
        for (int w = 0; w < team; ++w) {
          x += s_part[team > 1 ? w : warp][lane];
          y += s_part[team > 1 ? w : warp][kAngChunk + lane];
        }
        const int d = sf.ang_d[c0 + lane];
        Gi[d] = sf.ang_pref[c0 + lane] * x;
        Gi[d + nsf] = sf.ang_pref[c0 + lane] * y;
      }
      if (team > 1) __syncthreads();
      else __syncwarp();
    }
    __syncwarp();
  }
}

template <typename T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    k_wacsf_bwd(int N, int cap, int capS, const int *__restrict__ cnt,
                const double4 *__restrict__ xyzr, const int *__restrict__ nj,
                const double4 *__restrict__ apos, const float4 *__restrict__ d32,
                const float *__restrict__ w32, const SFT<T> *__restrict__ sfg,
                const T *__restrict__ dedg, typename Vec4<T>::type *__restrict__ gslot,
                double *__restrict__ wvir, int team) {
  using V4 = typename Vec4<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  load_table<T>(smraw, sfg);
  const SFT<T> &sf = *reinterpret_cast<const SFT<T> *>(smraw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nrc = sf.nrc, nal = sf.nalpha, D = sf.D, nsf = sf.nsf;
  const int nrad = sf.nrad, nang = sf.nang, ngrp = sf.n_ang_grp;
  const Layout<T> L = carve<T>(smraw, warp, capS, nrc, nal, D, nang, false);
  const T maxrc = sf.max_ang_rc;
  // The rounds fall into kTeam parts (part w: rounds w, w + kTeam, ...), each
  // summed into slot-gradient arrays of its own and the parts added in order.
  // team > 1: the block's warps share one atom and run one part each (warp
  // 0's arrays also hold the radial terms), added in warp order before warp 0
  // writes the slot gradients and the virial.  team = 1: the warp runs the
  // parts in turn, part 0 into its arrays and each later part into the
  // atom's row of gslot (global scratch until the final slot gradients are
  // written there), added after it.  The rounding is the same for every
  // launch shape.
  const int tw = team > 1 ? warp : 0;
  const int per_block = team > 1 ? 1 : kWarpsPerBlock;
  for (int i = blockIdx.x * per_block + (team > 1 ? 0 : warp); i < N; i += gridDim.x * per_block) {
    const int P = stage_slots<T>(L, sf, i, cap, capS, lane, cnt, xyzr, nj, apos, d32, w32, true);
    for (int d = lane; d < D; d += 32) L.dg[d] = dedg[(size_t)i * D + d];
    for (int q = lane; q < P; q += 32) L.gx[q] = L.gy[q] = L.gz[q] = (T)0;
    __syncwarp();
    // per-atom angular coefficients: 2^(1-zeta) dE/dG of both copies
    for (int s = lane; s < nang; s += 32) {
      const int d = sf.ang_d[s];
      L.cA[s] = sf.ang_pref[s] * L.dg[d];
      L.cB[s] = sf.ang_pref[s] * L.dg[d + nsf];
    }
    // radial terms: lanes own slots (the team's first warp)
    for (int q = lane; q < P && tw == 0; q += 32) {
      const T r = L.r[q], w = L.w[q];
      T S = (T)0;
      for (int s = 0; s < nrad; ++s) {
        const int rci = sf.rad_rc[s];
        if (r > sf.rc_val[rci]) continue;
        const T f = L.fc[(size_t)rci * capS + q], df = L.dfc[(size_t)rci * capS + q];
        const T alpha = sf.rad_alpha[s];
        const T u = r - sf.rad_rs[s];
        const T ex = t_exp(-alpha * u * u);
        const T dphi = (T)-2 * alpha * u * ex * f + ex * df;
        const int d = sf.rad_d[s];
        S += (L.dg[d] + L.dg[d + nsf] * w) * dphi;
      }
      const T ir = S / r;
      L.gx[q] += ir * L.dx[q];
      L.gy[q] += ir * L.dy[q];
      L.gz[q] += ir * L.dz[q];
    }
    __syncwarp();
    // angular terms in round-robin rounds (circle method over Pp slots)
    if (nang > 0 && P > 1) {
      const int Pp = P + (P & 1);
      const int half = Pp >> 1;
      const int part0 = team > 1 ? tw : 0, part1 = team > 1 ? tw + 1 : kTeam;
      for (int part = part0; part < part1; ++part) {
      const bool own = team > 1 || part == 0;
      V4 *tmp = gslot + (size_t)i * cap;  // this part's scratch when !own
      if (!own) {
        for (int q = lane; q < P; q += 32) {
          V4 z;
          z.x = z.y = z.z = z.w = (T)0;
          tmp[q] = z;
        }
        __syncwarp();
      }
      auto add = [&](int q, T vx, T vy, T vz) {
        if (own) {
          L.gx[q] += vx;
          L.gy[q] += vy;
          L.gz[q] += vz;
        } else {
          tmp[q].x += vx;
          tmp[q].y += vy;
          tmp[q].z += vz;
        }
      };
      for (int round = part; round < Pp - 1; round += kTeam) {
        for (int t = lane; t < half; t += 32) {
          int j, k;
          if (t == 0) {
            j = Pp - 1;
            k = round;
          } else {  // (round +- t) mod (Pp - 1) with 0 < t < Pp/2, round < Pp - 1
            j = round + t;
            if (j >= Pp - 1) j -= Pp - 1;
            k = round - t;
            if (k < 0) k += Pp - 1;
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
          for (int al = 0; al < nal; ++al)
            L.Ep[al * 32 + lane] = L.ea[(size_t)al * capS + j] * L.ea[(size_t)al * capS + k] *
                                   t_exp(-sf.alpha_val[al] * c2);
          const T wjk = L.w[j] * L.w[k];
          T S1 = (T)0, S2 = (T)0, S3 = (T)0;
          for (int g = 0; g < ngrp; ++g) {
            const int rci = sf.ang_grp_rc[g];
            if (a > sf.rc_val[rci] || b > sf.rc_val[rci] || c > sf.rc_val[rci]) continue;
            const T fa = L.fc[(size_t)rci * capS + j], fb = L.fc[(size_t)rci * capS + k];
            const T dfa = L.dfc[(size_t)rci * capS + j], dfb = L.dfc[(size_t)rci * capS + k];
            T sn, cs;
            t_sincos(sf.pi_over_rc[rci] * c, &sn, &cs);
            const T fcc = (T)0.5 * (cs + (T)1);
            const T dfcc = (T)-0.5 * sn * sf.pi_over_rc[rci];
            const T F = fa * fb * fcc;
            T SP = (T)0, SQ = (T)0, SU = (T)0;
            for (int s = sf.ang_grp_start[g]; s < sf.ang_grp_start[g + 1]; ++s) {
              const int code = sf.ang_code[s];
              const int al = (code >> 8) & 255, iz = (code >> 16) & 255;
              const T lam = (code >> 24) ? (T)-1 : (T)1;
              T A, dA;
              ang_pow<T>((T)1 + lam * cosv, iz, iz ? (T)1 : sf.ang_zeta[s], &A, &dA);
              const T X = (L.cA[s] + L.cB[s] * wjk) * L.Ep[al * 32 + lane];
              const T XA = X * A;
              SP += X * dA * lam;
              SQ += XA;
              SU += XA * sf.alpha_val[al];
            }
            // dG/da = E [A' dcos/da F + A (-2 alpha a F + fc'(a) fc(b) fc(c))], etc.
            S1 += F * (SP * dcda - (T)2 * SU * a) + SQ * (dfa * fb * fcc);
            S2 += F * (SP * dcdb - (T)2 * SU * b) + SQ * (fa * dfb * fcc);
            S3 += F * (SP * dcdc - (T)2 * SU * c) + SQ * (fa * fb * dfcc);
          }
          const T s1 = S1 * ia, s2 = S2 * ib, s3 = S3 * ic;
          add(j, s1 * djx + s3 * cx, s1 * djy + s3 * cy, s1 * djz + s3 * cz);
          add(k, s2 * dkx - s3 * cx, s2 * dky - s3 * cy, s2 * dkz - s3 * cz);
        }
        __syncwarp();
      }
      if (!own) {
        __syncwarp();
        for (int q = lane; q < P; q += 32) {
          const V4 t = tmp[q];
          L.gx[q] += t.x;
          L.gy[q] += t.y;
          L.gz[q] += t.z;
        }
        __syncwarp();
      }
      }
    }
    __syncwarp();
    if (team > 1) {
      __syncthreads();
      const Layout<T> L0 = carve<T>(smraw, 0, capS, nrc, nal, D, nang, false);
      for (int q = threadIdx.x; q < P; q += blockDim.x) {
        T gx = L0.gx[q], gy = L0.gy[q], gz = L0.gz[q];
        for (int w = 1; w < team; ++w) {
          const Layout<T> Lw = carve<T>(smraw, w, capS, nrc, nal, D, nang, false);
          gx += Lw.gx[q];
          gy += Lw.gy[q];
          gz += Lw.gz[q];
        }
        L0.gx[q] = gx;
        L0.gy[q] = gy;
        L0.gz[q] = gz;
      }
      __syncthreads();
      if (warp != 0) continue;
    }
    // slot gradients and the per-atom virial (lanes in T, the warp sum in FP64)
    T W[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = lane; q < P; q += 32) {
      const T gx = L.gx[q], gy = L.gy[q], gz = L.gz[q];
      V4 v;
      v.x = gx;
      v.y = gy;
      v.z = gz;
      v.w = (T)0;
      gslot[(size_t)i * cap + q] = v;
      const T d3[3] = {L.dx[q], L.dy[q], L.dz[q]};
      const T g3[3] = {gx, gy, gz};
#pragma unroll
      for (int aa = 0; aa < 3; ++aa)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) W[aa * 3 + bb] += d3[aa] * g3[bb];
    }
    double Wd[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) Wd[t] = warp_sum<double>((double)W[t]);
    if (lane < 9) {
      double v = 0;
#pragma unroll
      for (int t = 0; t < 9; ++t)
        if (lane == t) v = Wd[t];
      wvir[(size_t)i * 9 + lane] = v;
    }
    __syncwarp();
  }
}

#include "wacsf_grouped.cuh"

int warp_grid(int N, size_t smem_per_block, const void *fn) {
  const int sms = device_sms();
  const int per_sm = kernel_occupancy(fn, 32 * kWarpsPerBlock, smem_per_block);
  int need = (N + kWarpsPerBlock - 1) / kWarpsPerBlock;
  int maxb = sms * per_sm;
  return need < maxb ? (need > 0 ? need : 1) : maxb;
}

// Launch shape of the generic kernels: a batch of fewer than 8 atoms per SM
// (a single drop-in structure, say) would occupy a few warps per SM, so each
// atom gets a whole block (team = its kWarpsPerBlock warps); otherwise one
// warp per atom.
int team_grid(int N, size_t smem_per_block, const void *fn, int *team) {
  const int sms = device_sms();
  if (N < 8 * sms) {
    *team = kWarpsPerBlock;
    const int per_sm = kernel_occupancy(fn, 32 * kWarpsPerBlock, smem_per_block);
    const int maxb = sms * (per_sm > 0 ? per_sm : 1);
    return N < maxb ? (N > 0 ? N : 1) : maxb;
  }
  *team = 1;
  return warp_grid(N, smem_per_block, fn);
}

}  // namespace

size_t wacsf_smem_bytes(const SFDev &t, int capS, bool fwd, size_t elem) {
  const size_t table = elem == 8 ? kTableBytes(sizeof(SFT<double>)) : kTableBytes(sizeof(SFT<float>));
  const size_t per = elem == 8 ? per_warp_elems<double>(capS, t.nrc, t.nalpha, t.D, t.nang, fwd)
                               : per_warp_elems<float>(capS, t.nrc, t.nalpha, t.D, t.nang, fwd);
  return table + per * elem * kWarpsPerBlock;
}

template <typename T>
static const SFT<T> *sft_of(const gapgb_model *m);
template <>
const SFT<double> *sft_of<double>(const gapgb_model *m) { return m->d_sft64; }
template <>
const SFT<float> *sft_of<float>(const gapgb_model *m) { return m->d_sft32; }

template <typename T>
void launch_wacsf_fwd(const gapgb_model *m, Workspace &ws, int N, int cap, int capS,
                      cudaStream_t st, int a0, int a1) {
  const size_t smem = wacsf_smem_bytes(m->sfh, capS, true, sizeof(T));
  if (a1 < 0) a1 = N;
  const int D = m->sfh.D;
  if (m->sfh.D > 2 * m->sfh.nsf || m->sfh.nrad + m->sfh.nang < m->sfh.nsf)
    cudaMemsetAsync((T *)ws.G + (size_t)a0 * D, 0, sizeof(T) * (size_t)(a1 - a0) * D,
                    st);  // never-written entries
  if constexpr (std::is_same<T, float>::value) {
    GrpFwd gf;
    GrpBwd gb;
    if (!m->generic_kernels && grouped_kernels(m->sft32h, &gf, &gb)) {
      const size_t smg = kTableBytes(sizeof(SFT<float>)) +
                         (size_t)kWarpsPerBlock * 4 *
                             grp_warp_floats(capS, m->sfh.nrc, m->sfh.D, m->sfh.nrad, true);
      kernel_smem((const void *)gf, (int)smg, true);
      const int n = a1 - a0;
      if (n <= 0) return;
      const int grid = warp_grid(n, smg, (const void *)gf);
      // atoms [a0, a1) through per-atom arrays offset to a0
      const int pcap = capS <= 256 ? kPairCap : 0;
      gf<<<grid, 32 * kWarpsPerBlock, smg, st>>>(
          n, cap, capS, ws.nbr_cnt + a0, ws.nbr_xyz, ws.nbr_j, ws.apos,
          ws.nbr_d32 + (size_t)a0 * cap, ws.nbr_w32 + (size_t)a0 * cap, m->d_sft32,
          (float *)ws.G + (size_t)a0 * D, ws.pairs + (size_t)a0 * kPairCap, ws.pair_cnt + a0,
          pcap);
      return;
    }
  }
  auto fn = k_wacsf_fwd<T>;
  kernel_smem((const void *)fn, (int)smem);
  int team = 1;
  const int grid = team_grid(N, smem, (const void *)fn, &team);
  fn<<<grid, 32 * kWarpsPerBlock, smem, st>>>(N, cap, capS, ws.nbr_cnt, ws.nbr_xyz, ws.nbr_j,
                                               ws.apos, ws.nbr_d32, ws.nbr_w32, sft_of<T>(m),
                                               (T *)ws.G, team);
}

bool bwd_scatters_forces(const gapgb_model *m) {
  GrpFwd gf;
  GrpBwd gb;
  return m->precision != GAPGB_PREC_FP64 && !m->generic_kernels &&
         grouped_kernels(m->sft32h, &gf, &gb);
}

template <typename T>
bool launch_wacsf_bwd(const gapgb_model *m, Workspace &ws, int N, int cap, int capS,
                      double *d_force, cudaStream_t st, int a0, int a1, bool zero_force) {
  const size_t smem = wacsf_smem_bytes(m->sfh, capS, false, sizeof(T));
  if (a1 < 0) a1 = N;
  if constexpr (std::is_same<T, float>::value) {
    GrpFwd gf;
    GrpBwd gb;
    if (!m->generic_kernels && grouped_kernels(m->sft32h, &gf, &gb)) {
      const size_t smg = kTableBytes(sizeof(SFT<float>)) +
                         (size_t)kWarpsPerBlock * 4 *
                             grp_warp_floats(capS, m->sfh.nrc, m->sfh.D, m->sfh.nrad, false);
      kernel_smem((const void *)gb, (int)smg, true);
      if (zero_force) cudaMemsetAsync(d_force, 0, sizeof(double) * 3 * (size_t)N, st);
      const int n = a1 - a0;
      if (n <= 0) return true;
      const int grid = warp_grid(n, smg, (const void *)gb);
      // atoms [a0, a1) through per-atom arrays offset to a0; the partner
      // indices (nbr_j) and the force array stay global
      const int D = m->sfh.D;
      const int pcap = capS <= 256 ? kPairCap : 0;
      gb<<<grid, 32 * kWarpsPerBlock, smg, st>>>(
          n, a0, cap, capS, ws.nbr_cnt + a0, ws.nbr_xyz, ws.nbr_j + (size_t)a0 * cap, ws.apos,
          ws.nbr_d32 + (size_t)a0 * cap, ws.nbr_w32 + (size_t)a0 * cap, m->d_sft32,
          (const float *)ws.dedg + (size_t)a0 * D, d_force, ws.wvir + (size_t)a0 * 9,
          ws.pairs + (size_t)a0 * kPairCap, ws.pair_cnt + a0, pcap, ws.d_flags);
      return true;  // forces scattered by the kernel
    }
  }
  auto fn = k_wacsf_bwd<T>;
  kernel_smem((const void *)fn, (int)smem);
  int team = 1;
  const int grid = team_grid(N, smem, (const void *)fn, &team);
  fn<<<grid, 32 * kWarpsPerBlock, smem, st>>>(N, cap, capS, ws.nbr_cnt, ws.nbr_xyz, ws.nbr_j,
                                               ws.apos, ws.nbr_d32, ws.nbr_w32, sft_of<T>(m),
                                               (const T *)ws.dedg,
                                               (typename Vec4<T>::type *)ws.gslot, ws.wvir, team);
  (void)d_force;
  return false;  // slot gradients in ws.gslot: launch_forces gathers them
}

template void launch_wacsf_fwd<double>(const gapgb_model *, Workspace &, int, int, int, cudaStream_t,
                                       int, int);
template void launch_wacsf_fwd<float>(const gapgb_model *, Workspace &, int, int, int, cudaStream_t,
                                      int, int);
template bool launch_wacsf_bwd<double>(const gapgb_model *, Workspace &, int, int, int, double *,
                                       cudaStream_t, int, int, bool);
template bool launch_wacsf_bwd<float>(const gapgb_model *, Workspace &, int, int, int, double *,
                                      cudaStream_t, int, int, bool);

}  // namespace gapgb
