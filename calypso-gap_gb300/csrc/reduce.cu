// reduce.cu - forces by gather, per-structure energy and virial stress.
//
// Reference: gappy/libgap/gap_calc.f90:152-154 (E = sum e_i), :172-185
// (F_j = -sum_i sum_d dedg(i,d) dxdy(d,i,j,:)), :188-203 (stress from
// strs, divided by volume and GPa2eVPang) and :221-226 (reorder to
// XX YY ZZ XY YZ ZX).
//
// With gslot[i][q] = sum_d dedg_id dG_id/dp_q (wacsf.cu) and translation
// invariance of G_i (dG_i/dr_i = -sum_q dG_i/dp_q):
//   F_j = sum_q gslot[j][q] - sum_{(i,q) : partner(i,q) = j} gslot[i][q]
// and the second sum is a gather over the reverse slots of j's own list,
// sum_q gslot[partner(j,q)][rev(j,q)].  Slots whose reverse pair did not
// survive the cutoff test (a last-bit difference of the two distances at
// exactly r = rcut) are listed as orphans and added afterwards.
#include <algorithm>

#include "gapgb_internal.h"

namespace gapgb {
namespace {

template <typename T>
__global__ void __launch_bounds__(128)
    k_forces(int N, int cap, const int *__restrict__ cnt, const int *__restrict__ nj,
             const int *__restrict__ rev, const typename Vec4<T>::type *__restrict__ gslot,
             double *__restrict__ force) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  // accumulation type: FP64 for the FP64 path, FP32 for the FP32 forms
  // (FP64 adds and conversions run on the narrow FP64 pipe; a per-atom force
  // is a sum of ~2P slot terms, far inside FP32's precision needs here)
  using A = T;
  for (int j = gw; j < N; j += nw) {
    const int P = cnt[j];
    A fx = 0, fy = 0, fz = 0;
    for (int q = lane; q < P; q += 32) {
      const size_t idx = (size_t)j * cap + q;
      const auto g = gslot[idx];
      fx += (A)g.x;
      fy += (A)g.y;
      fz += (A)g.z;
      const int r = rev[idx];
      if (r >= 0) {
        const auto h = gslot[(size_t)nj[idx] * cap + r];
        fx -= (A)h.x;
        fy -= (A)h.y;
        fz -= (A)h.z;
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      fx += __shfl_xor_sync(0xffffffffu, fx, off);
      fy += __shfl_xor_sync(0xffffffffu, fy, off);
      fz += __shfl_xor_sync(0xffffffffu, fz, off);
    }
    if (lane == 0) {
      force[(size_t)j * 3 + 0] = (double)fx;
      force[(size_t)j * 3 + 1] = (double)fy;
      force[(size_t)j * 3 + 2] = (double)fz;
    }
  }
}

template <typename T>
__global__ void k_orphans(int cap, const int *__restrict__ flags, const int *__restrict__ orphans,
                          int orphan_cap, const int *__restrict__ nj,
                          const typename Vec4<T>::type *__restrict__ gslot,
                          double *__restrict__ force) {
  const int n = min(flags[2], orphan_cap);
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < n; o += gridDim.x * blockDim.x) {
    const int idx = orphans[o];
    const int j = nj[idx];
    const auto g = gslot[idx];
    atomicAdd(force + (size_t)j * 3 + 0, -(double)g.x);
    atomicAdd(force + (size_t)j * 3 + 1, -(double)g.y);
    atomicAdd(force + (size_t)j * 3 + 2, -(double)g.z);
  }
}

// Per-structure sums of e_i and the virial in two fixed-order stages: block
// (p, s) reduces part p of structure s's atoms (parts chosen from the batch
// shape, so that a single large cell spreads over many SMs; FP64 adds are
// slow on this part), then one thread per structure adds its parts in order.
constexpr int kMaxParts = 64;

__global__ void __launch_bounds__(128)
    k_struct_partial(int parts, int lgrad, const StructInfo *__restrict__ sinfo,
                     const double *__restrict__ e, const double *__restrict__ wvir,
                     double *__restrict__ atom_e, double *__restrict__ part) {
  __shared__ double red[7][128];
  const int s = blockIdx.y, p = blockIdx.x;
  const int a0 = sinfo[s].a0, na = sinfo[s].na;
  const int len = (na + parts - 1) / parts;
  const int beg = p * len, end = min(na, beg + len);
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  // upper triangle (a <= b) in the reference's k1 order: 11 12 13 22 23 33
  const int comp[6] = {0, 1, 2, 4, 5, 8};
  for (int q = beg + threadIdx.x; q < end; q += blockDim.x) {
    const int i = a0 + q;
    acc[0] += e[i];
    if (atom_e) atom_e[i] = e[i];
    if (lgrad)
      for (int c = 0; c < 6; ++c) acc[1 + c] += wvir[(size_t)i * 9 + comp[c]];
  }
  for (int c = 0; c < 7; ++c) red[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int c = 0; c < 7; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 7) part[((size_t)s * parts + p) * 7 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_struct_final(int S, int parts, int lgrad, const StructInfo *__restrict__ sinfo,
                               const double *__restrict__ part, double *__restrict__ energy,
                               double *__restrict__ stress) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int p = 0; p < parts; ++p)
    for (int c = 0; c < 7; ++c) v[c] += part[((size_t)s * parts + p) * 7 + c];
  energy[s] = v[0];
  double sc[6];
  const double vol = sinfo[s].volume;
  for (int c = 0; c < 6; ++c) sc[c] = lgrad ? -v[1 + c] * (1.0 / kGPa2eVPang) / vol : 0.0;
  double *o = stress + (size_t)s * 6;
  o[0] = sc[0];  // XX
  o[1] = sc[3];  // YY
  o[2] = sc[5];  // ZZ
  o[3] = sc[1];  // XY
  o[4] = sc[4];  // YZ
  o[5] = sc[2];  // ZX
}

}  // namespace

template <typename T>
void launch_forces(Workspace &ws, int N, int cap, double *d_force, cudaStream_t st) {
  using V4 = typename Vec4<T>::type;
  const int sms = device_sms();
  int blocks = (N + 3) / 4;
  if (blocks > sms * 16) blocks = sms * 16;
  if (blocks < 1) blocks = 1;
  k_forces<T><<<blocks, 128, 0, st>>>(N, cap, ws.nbr_cnt, ws.nbr_j, ws.nbr_rev,
                                       (const V4 *)ws.gslot, d_force);
  k_orphans<T><<<8, 128, 0, st>>>(cap, ws.d_flags, ws.orphans, ws.orphan_cap, ws.nbr_j,
                                   (const V4 *)ws.gslot, d_force);
}

void launch_struct_reduce(Workspace &ws, int S, int lgrad, double *d_energy, double *d_stress,
                          double *d_atom_e, int N, cudaStream_t st) {
  // about 2048 atoms per part for the mean structure size, at most kMaxParts
  const long per = S > 0 ? (long)N / S : 0;
  const int parts = (int)std::max(1L, std::min((long)kMaxParts, per / 2048));
  k_struct_partial<<<dim3(parts, S), 128, 0, st>>>(parts, lgrad, ws.sinfo, ws.e, ws.wvir,
                                                    d_atom_e, ws.red_part);
  k_struct_final<<<(S + 127) / 128, 128, 0, st>>>(S, parts, lgrad, ws.sinfo, ws.red_part,
                                                   d_energy, d_stress);
}

template void launch_forces<double>(Workspace &, int, int, double *, cudaStream_t);
template void launch_forces<float>(Workspace &, int, int, double *, cudaStream_t);

}  // namespace gapgb
