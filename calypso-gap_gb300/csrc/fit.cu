// fit.cu - sparse-GPR coefficients from training energies, on the device.
//
// The reference evaluates E = sum_i sum_k c_k K(x_i, m_k) (GET_COV and the
// energy sum of FGAP_CALC, gappy/libgap/gap_calc.f90:143-154, 268-288) with
// coefficients fitted elsewhere (calypso.x / ngap.x, not part of the
// repository).  This file fits them from structure energies, and optionally
// forces, with the sparse (subset-of-regressors) normal equations:
//   Phi_sk = sum_{i in s} K(x_i, m_k)                  (structure design rows)
//   PhiF_rk = force component r of the model with c = e_k  (force design rows)
//   PhiS_rk = stress component r (GPa) of the model with c = e_k  (stress rows)
//   A      = K_MM + jitter I + sum_s w_s Phi_s^T Phi_s + PhiF^T PhiF / sigma_f^2
//            + PhiS^T PhiS / sigma_s^2
//   b      = sum_s w_s Phi_s^T E_s + PhiF^T F / sigma_f^2 + PhiS^T sigma / sigma_s^2,
//   w_s = 1 / (sigma_e^2 n_s)
//   A c = b                                           (Cholesky, FP64)
// sigma_e is a per-atom energy noise (independent per atom, so a structure of
// n_s atoms has variance n_s sigma_e^2).  Everything is FP64: A inherits
// K_MM's conditioning.
//
// Force column k runs the FP64 gradient kernel and the force gather on the
// dE/dG of the unit coefficient e_k (M passes over the training atoms).
// Kernels: the design rows with the structure sum fused in (no N x M
// buffer), a tiled FP64 Gram product, a blocked right-looking Cholesky
// (64-wide diagonal factor in shared memory, row-parallel triangular solve
// of the panel, tiled update of the trailing lower triangle) and a
// single-CTA pair of triangular solves.  No kernel waits on another CTA.
#include <algorithm>
#include <string>
#include <vector>

#include "gapgb_internal.h"

namespace gapgb {
namespace {

constexpr int kT = 64;    // tile / block width
constexpr int kDC = 32;   // descriptor chunk staged in shared memory
constexpr int kRowsPerPass = 32;  // atoms per pass of the design-row kernel
constexpr int kKC = 16;   // contraction chunk of the tiled products

// Phi[s][k] = sum over structure s's atoms of exp(-1/2 |x_i / theta - m_k / theta|^2);
// structure s = atoms [off[s], off[s+1]) of the rows of G.  Block (k tile, s);
// zero for padded columns.
__global__ void __launch_bounds__(256)
    k_fit_phi(int M, int Mp, int D, const int *__restrict__ off, const double *__restrict__ G,
              const double *__restrict__ invth, const double *__restrict__ mmt,
              double *__restrict__ phi) {
  __shared__ double xs[kRowsPerPass][kDC + 1];
  __shared__ double ms[kT][kDC + 1];
  __shared__ double red[4][kT];
  const int tid = threadIdx.x, tx = tid & 63, ty = tid >> 6;
  const int s = blockIdx.y, kb = blockIdx.x * kT, k = kb + tx;
  const int a0 = off[s], a1 = off[s + 1];
  double sum = 0.0;
  for (int r0 = a0; r0 < a1; r0 += kRowsPerPass) {
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    for (int d0 = 0; d0 < D; d0 += kDC) {
      for (int e = tid; e < kRowsPerPass * kDC; e += 256) {
        const int r = e / kDC, d = d0 + e % kDC, i = r0 + r;
        xs[r][e % kDC] = (i < a1 && d < D) ? G[(size_t)i * D + d] * invth[d] : 0.0;
      }
      for (int e = tid; e < kT * kDC; e += 256) {
        const int kk = kb + e / kDC, d = d0 + e % kDC;
        ms[e / kDC][e % kDC] = (kk < M && d < D) ? mmt[(size_t)kk * D + d] : 0.0;
      }
      __syncthreads();
#pragma unroll 4
      for (int d = 0; d < kDC; ++d) {
        const double mv = ms[tx][d];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const double t = xs[ty + 4 * q][d] - mv;
          acc[q] += t * t;
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (r0 + ty + 4 * q < a1) sum += exp(-0.5 * acc[q]);
  }
  red[ty][tx] = sum;
  __syncthreads();
  if (ty == 0) {
    const double v = ((red[0][tx] + red[1][tx]) + red[2][tx]) + red[3][tx];
    phi[(size_t)s * Mp + k] = k < M ? v : 0.0;
  }
}

// K_MM[r][k] = exp(-1/2 |m_r / theta - m_k / theta|^2) into A (rows < M; zero
// for padded columns).  Block (k tile, 32-row tile).
__global__ void __launch_bounds__(256)
    k_fit_kmm(int M, int Mp, int D, const double *__restrict__ mmt, double *__restrict__ A) {
  __shared__ double xs[kRowsPerPass][kDC + 1];
  __shared__ double ms[kT][kDC + 1];
  const int tid = threadIdx.x, tx = tid & 63, ty = tid >> 6;
  const int rb = blockIdx.y * kRowsPerPass, kb = blockIdx.x * kT;
  double acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = 0.0;
  for (int d0 = 0; d0 < D; d0 += kDC) {
    for (int e = tid; e < kRowsPerPass * kDC; e += 256) {
      const int r = rb + e / kDC, d = d0 + e % kDC;
      xs[e / kDC][e % kDC] = (r < M && d < D) ? mmt[(size_t)r * D + d] : 0.0;
    }
    for (int e = tid; e < kT * kDC; e += 256) {
      const int k = kb + e / kDC, d = d0 + e % kDC;
      ms[e / kDC][e % kDC] = (k < M && d < D) ? mmt[(size_t)k * D + d] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int d = 0; d < kDC; ++d) {
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
    if (r < M) A[(size_t)r * Mp + k] = k < M ? exp(-0.5 * acc[q]) : 0.0;
  }
}

// A[r][c] (lower tiles only) = base[r][c] + sum_s w_s Phi_sr Phi_sc, and the
// padded diagonal set to 1; base = K_MM + jitter I (in A already).  Block
// (c tile, r tile) with c tile <= r tile.
__global__ void __launch_bounds__(256)
    k_fit_gram(int S, int M, int Mp, const double *__restrict__ phi, const double *__restrict__ w,
               double *__restrict__ A) {
  const int rt = blockIdx.y, ct = blockIdx.x;
  if (ct > rt) return;
  __shared__ double Rs[kKC][kT + 1];
  __shared__ double Cs[kKC][kT + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int rb = rt * kT, cb = ct * kT;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int s0 = 0; s0 < S; s0 += kKC) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = tid + 256 * q, ss = e / kT, j = e % kT, s = s0 + ss;
      const bool live = s < S;
      const double ws = live ? w[s] : 0.0;
      Rs[ss][j] = live ? phi[(size_t)s * Mp + rb + j] * ws : 0.0;
      Cs[ss][j] = live ? phi[(size_t)s * Mp + cb + j] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int ss = 0; ss < kKC; ++ss) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = Rs[ss][ty * 4 + u];
        b[u] = Cs[ss][tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int r = rb + ty * 4 + u, c = cb + tx * 4 + v;
      double *p = A + (size_t)r * Mp + c;
      if (r >= M || c >= M) *p = (r == c) ? 1.0 : 0.0;
      else *p += acc[u][v];
    }
}

// b[k] += sum_s w_s Phi_sk E_s (fixed order over s)
__global__ void k_fit_rhs(int S, int Mp, const double *__restrict__ phi,
                          const double *__restrict__ w, const double *__restrict__ E,
                          double *__restrict__ b) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= Mp) return;
  double acc = 0.0;
  for (int s = 0; s < S; ++s) acc = fma(w[s] * E[s], phi[(size_t)s * Mp + k], acc);
  b[k] += acc;
}

// dE/dG of the model with c = e_k (one sparse point, unit coefficient), the
// loop of gap_calc.f90:157-166 for one k:
//   dedg_id = -K_ik (x_id - m_kd) / theta_d^2,  K_ik = exp(-1/2 sum_d ((x_id - m_kd)/theta_d)^2)
// one warp per atom
__global__ void __launch_bounds__(128)
    k_fit_dedg_unit(int N, int D, int k, const double *__restrict__ G,
                    const double *__restrict__ invth, const double *__restrict__ mmt,
                    double *__restrict__ dedg) {
  const int lane = threadIdx.x & 31;
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= N) return;
  double q[4];
  double s = 0.0;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int d = lane + 32 * t;
    q[t] = d < D ? G[(size_t)i * D + d] * invth[d] - mmt[(size_t)k * D + d] : 0.0;
    s += q[t] * q[t];
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  const double K = exp(-0.5 * s);
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int d = lane + 32 * t;
    if (d < D) dedg[(size_t)i * D + d] = -K * q[t] * invth[d];
  }
}

// column k of the force design matrix: PhiF[r][k] = F_r for the unit coefficient
__global__ void k_fit_col(int R, int k, int Mp, const double *__restrict__ F,
                          double *__restrict__ PhiF) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < R) PhiF[(size_t)r * Mp + k] = F[r];
}

__global__ void k_fit_fill(int n, double v, double *__restrict__ x) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) x[r] = v;
}

__global__ void k_fit_weights(int S, const int *__restrict__ off, double inv_var,
                              double *__restrict__ w) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < S) w[s] = inv_var / (double)max(1, off[s + 1] - off[s]);
}

__global__ void k_fit_jitter(int M, int Mp, double jitter, double *__restrict__ A) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < M) A[(size_t)k * Mp + k] += jitter;
}

// ---- blocked Cholesky, lower, row-major, in place --------------------------

// the 64 x 64 diagonal block at (j0, j0): unblocked Cholesky in shared memory
__global__ void __launch_bounds__(256)
    k_chol_diag(int Mp, int j0, double *__restrict__ A, int *__restrict__ flags) {
  __shared__ double T[kT][kT + 1];
  const int tid = threadIdx.x;
  for (int e = tid; e < kT * kT; e += 256) {
    const int r = e / kT, c = e % kT;
    T[r][c] = A[(size_t)(j0 + r) * Mp + j0 + c];
  }
  __syncthreads();
  for (int c = 0; c < kT; ++c) {
    if (tid == 0) {
      double d = T[c][c];
      if (!(d > 0.0)) {  // not positive definite: flag it, keep going on a floor
        atomicOr(flags, kFlagNotPositiveDefinite);
        d = 1e-300;
      }
      T[c][c] = sqrt(d);
    }
    __syncthreads();
    const double inv = 1.0 / T[c][c];
    for (int r = c + 1 + tid; r < kT; r += 256) T[r][c] *= inv;
    __syncthreads();
    // trailing update of the block's lower triangle: rows r > c, cols c < l <= r
    const int n = kT - 1 - c;
    for (int e = tid; e < n * n; e += 256) {
      const int r = c + 1 + e / n, l = c + 1 + e % n;
      if (l <= r) T[r][l] -= T[r][c] * T[l][c];
    }
    __syncthreads();
  }
  for (int e = tid; e < kT * kT; e += 256) {
    const int r = e / kT, c = e % kT;
    if (c <= r) A[(size_t)(j0 + r) * Mp + j0 + c] = T[r][c];
  }
}

// rows below the diagonal block: L[i][j0:j0+64] = A[i][j0:j0+64] L_jj^-T
// (forward substitution, one thread per row)
__global__ void __launch_bounds__(128)
    k_chol_panel(int Mp, int j0, double *__restrict__ A) {
  __shared__ double L[kT][kT + 1];
  const int tid = threadIdx.x;
  for (int e = tid; e < kT * kT; e += 128) {
    const int r = e / kT, c = e % kT;
    L[r][c] = c <= r ? A[(size_t)(j0 + r) * Mp + j0 + c] : 0.0;
  }
  __syncthreads();
  const int i = j0 + kT + blockIdx.x * 128 + tid;
  if (i >= Mp) return;
  double *row = A + (size_t)i * Mp + j0;
  double x[kT];
#pragma unroll
  for (int c = 0; c < kT; ++c) {
    double v = row[c];
#pragma unroll
    for (int q = 0; q < c; ++q) v = fma(-x[q], L[c][q], v);
    x[c] = v / L[c][c];
  }
#pragma unroll
  for (int c = 0; c < kT; ++c) row[c] = x[c];
}

// trailing update: A[r][c] -= sum_{q < 64} L[r][j0+q] L[c][j0+q] for the
// lower tiles of rows / columns >= j0 + 64.  blockIdx.x enumerates the
// (row tile, col tile <= row tile) pairs.
__global__ void __launch_bounds__(256)
    k_chol_update(int Mp, int j0, double *__restrict__ A) {
  int t = blockIdx.x, rt = 0;
  while (t > rt) {  // row tile rt holds rt + 1 column tiles
    t -= rt + 1;
    ++rt;
  }
  const int ct = t;
  const int base = j0 + kT;
  const int rb = base + rt * kT, cb = base + ct * kT;
  __shared__ double Rs[kKC][kT + 1];
  __shared__ double Cs[kKC][kT + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
  for (int q0 = 0; q0 < kT; q0 += kKC) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = tid + 256 * q, j = e / kKC, kk = e % kKC;
      Rs[kk][j] = A[(size_t)(rb + j) * Mp + j0 + q0 + kk];
      Cs[kk][j] = A[(size_t)(cb + j) * Mp + j0 + q0 + kk];
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKC; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = Rs[kk][ty * 4 + u];
        b[u] = Cs[kk][tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int r = rb + ty * 4 + u, c = cb + tx * 4 + v;
      if (c <= r) A[(size_t)r * Mp + c] -= acc[u][v];
    }
}

// L y = b then L^T c = y, one CTA of 1024 threads: per 64-row block the
// contributions of the finished blocks are summed by 16 threads per row (fixed
// order), then one thread substitutes within the block
__global__ void __launch_bounds__(1024)
    k_chol_solve(int Mp, const double *__restrict__ A, const double *__restrict__ b,
                 double *__restrict__ y, double *__restrict__ c) {
  __shared__ double part[kT][17];
  __shared__ double blk[kT];
  const int tid = threadIdx.x, rr = tid >> 4, lane16 = tid & 15;
  // forward
  for (int j0 = 0; j0 < Mp; j0 += kT) {
    const int r = j0 + rr;
    double p = 0.0;
    for (int k = lane16; k < j0; k += 16) p = fma(A[(size_t)r * Mp + k], y[k], p);
    part[rr][lane16] = p;
    __syncthreads();
    if (tid < kT) {
      double v = 0.0;
      for (int q = 0; q < 16; ++q) v += part[tid][q];
      blk[tid] = b[j0 + tid] - v;
    }
    __syncthreads();
    if (tid == 0)
      for (int q = 0; q < kT; ++q) {
        double v = blk[q];
        for (int t = 0; t < q; ++t) v = fma(-A[(size_t)(j0 + q) * Mp + j0 + t], y[j0 + t], v);
        y[j0 + q] = v / A[(size_t)(j0 + q) * Mp + j0 + q];
      }
    __syncthreads();
  }
  // backward: c_r = (y_r - sum_{k > r} L[k][r] c_k) / L[r][r]
  for (int j0 = Mp - kT; j0 >= 0; j0 -= kT) {
    const int r = j0 + rr;
    double p = 0.0;
    for (int k = j0 + kT + lane16; k < Mp; k += 16) p = fma(A[(size_t)k * Mp + r], c[k], p);
    part[rr][lane16] = p;
    __syncthreads();
    if (tid < kT) {
      double v = 0.0;
      for (int q = 0; q < 16; ++q) v += part[tid][q];
      blk[tid] = y[j0 + tid] - v;
    }
    __syncthreads();
    if (tid == 0)
      for (int q = kT - 1; q >= 0; --q) {
        double v = blk[q];
        for (int t = q + 1; t < kT; ++t) v = fma(-A[(size_t)(j0 + t) * Mp + j0 + q], c[j0 + t], v);
        c[j0 + q] = v / A[(size_t)(j0 + q) * Mp + j0 + q];
      }
    __syncthreads();
  }
}

template <typename T>
gapgb_status dev_alloc(T **p, size_t n) {
  if (cudaMalloc(p, n * sizeof(T)) != cudaSuccess) {
    set_last_error("cudaMalloc of " + std::to_string(n * sizeof(T)) + " bytes for the fit failed");
    return GAPGB_ERR_CUDA;
  }
  return GAPGB_OK;
}

}  // namespace

// Fits the coefficients from FP64 descriptors d_G[N][D] (structures by
// d_off, S + 1 offsets on the device), host energies[S] and, when forces is
// not null, host forces[N][3] (the neighbour list of the descriptors, built
// with capacity cap and slot count capS, must still be in the workspace);
// writes the M coefficients to host coeff.  Synchronises the stream.
gapgb_status fit_enqueue(gapgb_model *m, int S, int N, int cap, int capS, const int *d_off,
                         const double *d_G, const double *energy, const double *forces,
                         const double *stress, double sigma_e, double sigma_f, double sigma_s,
                         double jitter, double *coeff, cudaStream_t st) {
  const int M = m->host.M, D = m->host.D, Mp = (M + kT - 1) / kT * kT;
  const int R = forces ? 3 * N : 0;   // force rows
  const int RS = stress ? 6 * S : 0;  // stress rows
  double *phi = nullptr, *A = nullptr, *b = nullptr, *y = nullptr, *c = nullptr, *w = nullptr,
         *E = nullptr, *phif = nullptr, *wf = nullptr, *Fv = nullptr, *Fk = nullptr,
         *phis = nullptr, *ws6 = nullptr, *Sv = nullptr, *Sk = nullptr, *Ek = nullptr;
  gapgb_status s = GAPGB_OK;
  auto cleanup = [&]() {
    for (double *p : {phi, A, b, y, c, w, E, phif, wf, Fv, Fk, phis, ws6, Sv, Sk, Ek})
      if (p) cudaFree(p);
  };
  if ((s = dev_alloc(&phi, (size_t)S * Mp)) || (s = dev_alloc(&A, (size_t)Mp * Mp)) ||
      (s = dev_alloc(&b, (size_t)Mp)) || (s = dev_alloc(&y, (size_t)Mp)) ||
      (s = dev_alloc(&c, (size_t)Mp)) || (s = dev_alloc(&w, (size_t)S)) ||
      (s = dev_alloc(&E, (size_t)S)) ||
      ((R > 0 || RS > 0) && ((s = dev_alloc(&Fk, (size_t)3 * N)) ||
                             (s = dev_alloc(&Sk, (size_t)6 * S)) ||
                             (s = dev_alloc(&Ek, (size_t)S)))) ||
      (R > 0 && ((s = dev_alloc(&phif, (size_t)R * Mp)) || (s = dev_alloc(&wf, (size_t)R)) ||
                 (s = dev_alloc(&Fv, (size_t)R)))) ||
      (RS > 0 && ((s = dev_alloc(&phis, (size_t)RS * Mp)) || (s = dev_alloc(&ws6, (size_t)RS)) ||
                  (s = dev_alloc(&Sv, (size_t)RS))))) {
    cleanup();
    return s;
  }
  auto tryc = [&](cudaError_t e) {
    if (e != cudaSuccess && s == GAPGB_OK) {
      set_last_error(std::string("fit: ") + cudaGetErrorString(e));
      s = GAPGB_ERR_CUDA;
    }
  };
  tryc(cudaMemcpyAsync(E, energy, sizeof(double) * S, cudaMemcpyHostToDevice, st));
  tryc(cudaMemsetAsync(A, 0, sizeof(double) * (size_t)Mp * Mp, st));
  tryc(cudaMemsetAsync(b, 0, sizeof(double) * (size_t)Mp, st));
  const int nt = Mp / kT;
  k_fit_kmm<<<dim3(nt, (M + kRowsPerPass - 1) / kRowsPerPass), 256, 0, st>>>(M, Mp, D, m->d_mmt, A);
  k_fit_jitter<<<(M + 255) / 256, 256, 0, st>>>(M, Mp, jitter, A);
  k_fit_weights<<<(S + 255) / 256, 256, 0, st>>>(S, d_off, 1.0 / (sigma_e * sigma_e), w);
  k_fit_phi<<<dim3(nt, S), 256, 0, st>>>(M, Mp, D, d_off, d_G, m->d_invth, m->d_mmt, phi);
  k_fit_gram<<<dim3(nt, nt), 256, 0, st>>>(S, M, Mp, phi, w, A);
  k_fit_rhs<<<(Mp + 255) / 256, 256, 0, st>>>(S, Mp, phi, w, E, b);
  if (R > 0 || RS > 0) {
    // force / stress rows: column k is the force field / stress of the unit
    // coefficient e_k, through the FP64 gradient kernel, the reverse-slot
    // gather and the structure sums
    Workspace &ws = m->ws;
    if (R > 0) {
      tryc(cudaMemcpyAsync(Fv, forces, sizeof(double) * R, cudaMemcpyHostToDevice, st));
      tryc(cudaMemsetAsync(phif, 0, sizeof(double) * (size_t)R * Mp, st));
      k_fit_fill<<<(R + 255) / 256, 256, 0, st>>>(R, 1.0 / (sigma_f * sigma_f), wf);
    }
    if (RS > 0) {
      tryc(cudaMemcpyAsync(Sv, stress, sizeof(double) * RS, cudaMemcpyHostToDevice, st));
      tryc(cudaMemsetAsync(phis, 0, sizeof(double) * (size_t)RS * Mp, st));
      k_fit_fill<<<(RS + 255) / 256, 256, 0, st>>>(RS, 1.0 / (sigma_s * sigma_s), ws6);
    }
    launch_reverse(ws, N, cap, st);
    for (int k = 0; k < M; ++k) {
      k_fit_dedg_unit<<<(N + 3) / 4, 128, 0, st>>>(N, D, k, d_G, m->d_invth, m->d_mmt,
                                                   (double *)ws.dedg);
      launch_wacsf_bwd<double>(m, ws, N, cap, capS, Fk, st);
      if (R > 0) {
        launch_forces<double>(ws, N, cap, Fk, st);
        k_fit_col<<<(R + 255) / 256, 256, 0, st>>>(R, k, Mp, Fk, phif);
      }
      if (RS > 0) {
        launch_struct_reduce(ws, S, 1, Ek, Sk, nullptr, N, st);
        k_fit_col<<<(RS + 255) / 256, 256, 0, st>>>(RS, k, Mp, Sk, phis);
      }
    }
    if (R > 0) {
      k_fit_gram<<<dim3(nt, nt), 256, 0, st>>>(R, M, Mp, phif, wf, A);
      k_fit_rhs<<<(Mp + 255) / 256, 256, 0, st>>>(R, Mp, phif, wf, Fv, b);
    }
    if (RS > 0) {
      k_fit_gram<<<dim3(nt, nt), 256, 0, st>>>(RS, M, Mp, phis, ws6, A);
      k_fit_rhs<<<(Mp + 255) / 256, 256, 0, st>>>(RS, Mp, phis, ws6, Sv, b);
    }
  }
  for (int j0 = 0; j0 < Mp; j0 += kT) {
    k_chol_diag<<<1, 256, 0, st>>>(Mp, j0, A, m->ws.d_flags);
    const int rest = Mp - j0 - kT;
    if (rest > 0) {
      k_chol_panel<<<(rest + 127) / 128, 128, 0, st>>>(Mp, j0, A);
      const int nr = rest / kT;
      k_chol_update<<<nr * (nr + 1) / 2, 256, 0, st>>>(Mp, j0, A);
    }
  }
  k_chol_solve<<<1, 1024, 0, st>>>(Mp, A, b, y, c);
  tryc(cudaGetLastError());
  tryc(cudaMemcpyAsync(coeff, c, sizeof(double) * M, cudaMemcpyDeviceToHost, st));
  tryc(cudaStreamSynchronize(st));
  cleanup();
  return s;
}

}  // namespace gapgb
