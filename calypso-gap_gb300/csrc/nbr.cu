// nbr.cu - structure/atom preparation and the periodic neighbour list.
//
// Reference: FGAP_CALC's image loop, gappy/libgap/gap_calc.f90:85-120.  For
// every atom i the reference visits j = 1..N, then n1, n2, n3 in
// [-nabc, nabc] ascending, forms xyz = pos(j) + n1 a1 + n2 a2 + n3 a3,
// dr = pos(i) - xyz, dis = sqrt(dr.dr) and keeps the image if dis <= rcut
// (self image (0,0,0) skipped).  Here one warp owns atom i and its lanes own
// consecutive j.  Each lane prunes its pair's image box with the
// fractional-coordinate bound |f_a + n_a| <= rcut*|b_a|/(2 pi) and screens
// the images in FP32 against rcut plus a rounding margin (both conservative).
// The survivors go, in the reference order (lane = j, then n1, n2, n3),
// through a per-warp shared queue, and the warp applies the reference's FP64
// distance test 32 candidates at a time (separately rounded operations in the
// reference's statement order), appending hits with a ballot prefix.  The
// kept set, its order and every stored distance are bit-identical to the loop
// above.
#include <algorithm>
#include <cfloat>

#include "gapgb_internal.h"

namespace gapgb {
namespace {

__device__ __forceinline__ void crossp_rn(const double *a, const double *b, double *o) {
  o[0] = __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1]));
  o[1] = __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(a[0], b[2]));
  o[2] = __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0]));
}

// One thread per structure: image counts (gap_calc.f90:85-88 with
// recipvector/volume/crossp of :240-266, same operation order), volume
// (det, :201 and :290-299) and the inverse lattice for pruning.
__global__ void k_prep_struct(int S, const int *__restrict__ atom_off,
                              const double *__restrict__ lat_all, double rcut, int allow_bins,
                              StructInfo *__restrict__ out, int *__restrict__ flags) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  StructInfo si;
  const double *L = lat_all + (size_t)s * 9;
  for (int q = 0; q < 9; ++q) si.lat[q] = L[q];
  // Fortran LAT(i,j) = L[(i-1)*3 + (j-1)]; columns c_j = LAT(:,j)
  double c1[3] = {L[0], L[3], L[6]}, c2[3] = {L[1], L[4], L[7]}, c3[3] = {L[2], L[5], L[8]};
  double r1[3], r2[3], r3[3];
  crossp_rn(c2, c3, r1);
  crossp_rn(c3, c1, r2);
  crossp_rn(c1, c2, r3);
  double vol = fabs(__dadd_rn(__dadd_rn(__dmul_rn(c1[0], r1[0]), __dmul_rn(c1[1], r1[1])),
                              __dmul_rn(c1[2], r1[2])));
  double *cols[3] = {r1, r2, r3};
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      cols[a][b] = __dmul_rn(__dmul_rn(__ddiv_rn(cols[a][b], vol), kPiRef), 2.0);
  for (int row = 0; row < 3; ++row) {
    double x = r1[row], y = r2[row], z = r3[row];
    double len = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
    double n = ceil(__ddiv_rn(__ddiv_rn(__dmul_rn(rcut, len), kPiRef), 2.0));
    if (!(n <= (double)kMaxImage)) {  // also catches NaN
      atomicOr(flags, kFlagImageLimit);
      n = (n > 0) ? (double)kMaxImage : 0.0;
    }
    si.nabc[row] = (int)n;
  }
  // det(lat) as gap_calc.f90:295-297
  double det = __dadd_rn(
      __dsub_rn(__dmul_rn(L[0], __dsub_rn(__dmul_rn(L[4], L[8]), __dmul_rn(L[5], L[7]))),
                __dmul_rn(L[1], __dsub_rn(__dmul_rn(L[3], L[8]), __dmul_rn(L[5], L[6])))),
      __dmul_rn(L[2], __dsub_rn(__dmul_rn(L[3], L[7]), __dmul_rn(L[6], L[4]))));
  si.volume = fabs(det);
  // inverse of L (rows = lattice vectors): adjugate / det
  double inv[9];
  inv[0] = (L[4] * L[8] - L[5] * L[7]) / det;
  inv[1] = (L[2] * L[7] - L[1] * L[8]) / det;
  inv[2] = (L[1] * L[5] - L[2] * L[4]) / det;
  inv[3] = (L[5] * L[6] - L[3] * L[8]) / det;
  inv[4] = (L[0] * L[8] - L[2] * L[6]) / det;
  inv[5] = (L[2] * L[3] - L[0] * L[5]) / det;
  inv[6] = (L[3] * L[7] - L[4] * L[6]) / det;
  inv[7] = (L[1] * L[6] - L[0] * L[7]) / det;
  inv[8] = (L[0] * L[4] - L[1] * L[3]) / det;
  for (int q = 0; q < 9; ++q) si.linv[q] = inv[q];
  for (int a = 0; a < 3; ++a) {
    double cl = sqrt(inv[a] * inv[a] + inv[3 + a] * inv[3 + a] + inv[6 + a] * inv[6 + a]);
    // FP32 fractional coordinates are compared against this bound: margin
    // for their rounding (|f| < 1e3 keeps the error below 1e-4)
    si.ext[a] = rcut * cl * (1.0 + 1e-9) + 2e-4;
  }
  {
    float lsum = 0.f;
    for (int q = 0; q < 9; ++q) {
      si.lat32[q] = (float)si.lat[q];
      si.latl32[q] = (float)(si.lat[q] - (double)si.lat32[q]);
      lsum += fabsf(si.lat32[q]);
    }
    const float rs = (float)rcut + 2.5e-4f * lsum + 1e-3f;
    si.r2max32 = rs * rs;
    si.rc2_32 = (float)(rcut * rcut);
    for (int a = 0; a < 3; ++a) si.ext32[a] = (float)si.ext[a];
    si.single = (2.f * si.ext32[0] < 1.f) & (2.f * si.ext32[1] < 1.f) & (2.f * si.ext32[2] < 1.f);
  }
  si.a0 = atom_off[s];
  si.na = atom_off[s + 1] - atom_off[s];
  // bins of fractional width >= ext (+ 1e-3 for the FP32 coordinates of the
  // binning) when the cell is at least 3 bins wide on every axis
  si.nb[0] = si.nb[1] = si.nb[2] = 0;
  si.bin0 = 0;
  if (allow_bins && si.na >= kBinMinAtoms) {
    int nb[3];
    bool ok = true;
    long prod = 1;
    for (int a = 0; a < 3; ++a) {
      nb[a] = (int)floor(1.0 / (si.ext[a] + 1e-3));
      if (nb[a] > 64) nb[a] = 64;
      if (nb[a] < 3) ok = false;
      prod *= nb[a];
    }
    if (ok && prod <= si.na)
      for (int a = 0; a < 3; ++a) si.nb[a] = nb[a];
  }
  // which of the two neighbour kernels has work (the other returns at once)
  if (si.nb[0] == 0) atomicOr(flags + (si.single ? 4 : 3), 1);
  out[s] = si;
}

// ---- spatial bins of large cells -------------------------------------------

// bin offsets of every binned structure and the total (one thread)
__global__ void k_bin_offsets(int S, StructInfo *__restrict__ sinfo, int *__restrict__ total) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int t = 0;
  for (int s = 0; s < S; ++s) {
    sinfo[s].bin0 = t;
    t += sinfo[s].nb[0] * sinfo[s].nb[1] * sinfo[s].nb[2];
  }
  *total = t;
}

// bin of every atom of a binned structure (from its wrapped FP32 fractional
// coordinates), its slot in the bin and its wrap shift m = floor(f)
__global__ void k_bin_count(int N, const float4 *__restrict__ frac32,
                            const int *__restrict__ atom_struct,
                            const StructInfo *__restrict__ sinfo, int *__restrict__ count,
                            int *__restrict__ atom_bin, int *__restrict__ atom_slot,
                            int *__restrict__ atom_m) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const StructInfo &si = sinfo[atom_struct[i]];
  if (si.nb[0] == 0) return;
  const float4 f = frac32[i];
  const float fv[3] = {f.x, f.y, f.z};
  int b[3], m[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float fl = floorf(fv[a]);
    m[a] = (int)fl;
    int bb = (int)((fv[a] - fl) * (float)si.nb[a]);
    b[a] = bb < 0 ? 0 : (bb >= si.nb[a] ? si.nb[a] - 1 : bb);
  }
  const int gid = si.bin0 + (b[0] * si.nb[1] + b[1]) * si.nb[2] + b[2];
  atom_bin[i] = gid;
  atom_slot[i] = atomicAdd(&count[gid], 1);
  atom_m[i] = ((m[0] + 128) << 16) | ((m[1] + 128) << 8) | (m[2] + 128);
}

// exclusive scan of the bin counts (one block)
__global__ void k_bin_scan(const int *__restrict__ total, const int *__restrict__ count,
                           int *__restrict__ start) {
  __shared__ int part[1024];
  const int T = *total;
  int carry = 0;
  for (int base = 0; base < T; base += 1024) {
    const int t = base + threadIdx.x;
    const int v = t < T ? count[t] : 0;
    part[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const int add = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
      __syncthreads();
      part[threadIdx.x] += add;
      __syncthreads();
    }
    if (t < T) start[t] = carry + part[threadIdx.x] - v;
    carry += part[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) start[T] = carry;
}

__global__ void k_bin_fill(int N, const int *__restrict__ atom_struct,
                           const StructInfo *__restrict__ sinfo, const int *__restrict__ atom_bin,
                           const int *__restrict__ atom_slot, const int *__restrict__ start,
                           int *__restrict__ bin_atoms) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (sinfo[atom_struct[i]].nb[0] == 0) return;
  bin_atoms[start[atom_bin[i]] + atom_slot[i]] = i;
}

// One thread per atom: structure index, species weight, fractional coords.
__global__ void k_prep_atoms(int N, int S, const int *__restrict__ atom_off,
                             const int *__restrict__ species, const double *__restrict__ pos,
                             const SFDev *__restrict__ sf, const StructInfo *__restrict__ sinfo,
                             int *__restrict__ atom_struct, double4 *__restrict__ apos,
                             float4 *__restrict__ frac32, float4 *__restrict__ pos2f,
                             int *__restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int lo = 0, hi = S;  // largest s with atom_off[s] <= i
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (atom_off[mid] <= i) lo = mid; else hi = mid;
  }
  atom_struct[i] = lo;
  int z = species[i];
  double w = 0.0;
  bool found = false;
  for (int q = 0; q < sf->nspecies; ++q)
    if (sf->species_z[q] == z) { w = sf->species_w[q]; found = true; }
  if (!found) atomicOr(flags, kFlagUnknownSpecies);
  double x = pos[3 * (size_t)i], y = pos[3 * (size_t)i + 1], zc = pos[3 * (size_t)i + 2];
  apos[i] = make_double4(x, y, zc, w);
  const float xh = (float)x, yh = (float)y, zh = (float)zc;
  pos2f[2 * (size_t)i] = make_float4(xh, yh, zh, 0.f);
  pos2f[2 * (size_t)i + 1] = make_float4((float)(x - (double)xh), (float)(y - (double)yh),
                                         (float)(zc - (double)zh), 0.f);
  const double *inv = sinfo[lo].linv;
  frac32[i] = make_float4((float)(x * inv[0] + y * inv[3] + zc * inv[6]),
                          (float)(x * inv[1] + y * inv[4] + zc * inv[7]),
                          (float)(x * inv[2] + y * inv[5] + zc * inv[8]), (float)w);
}

// Reference distance of image (n1,n2,n3) of atom j from atom i, with the
// reference's operation order and no contraction (gap_calc.f90:98-100).
// IEEE double -> float with round-to-nearest-even, in integer arithmetic so
// that it stays off the narrow FP64 pipe.  For finite |v| below 2^128;
// results below the float normal range become a signed zero (distances and
// relative vectors here are either zero or far above 1e-38).
__device__ __forceinline__ float d2f_rn(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
  if (e <= 0) return __uint_as_float(sign);
  const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  const unsigned m = (unsigned)(mant >> 29);
  const unsigned long long rem = mant & 0x1FFFFFFFull;
  unsigned r = ((unsigned)e << 23) | m;
  if (rem > 0x10000000ull || (rem == 0x10000000ull && (m & 1u))) r += 1u;  // carry is exact
  return __uint_as_float(sign | r);
}

// `dn` holds the image indices as doubles (exactly (double)n; read from a
// table instead of converted, since int-to-double conversion occupies the
// narrow FP64 pipe).
__device__ __forceinline__ double ref_image(const double4 &pi, const double4 &pj,
                                            const double *L, double dn1, double dn2, double dn3,
                                            double *xyz) {
  const double p[3] = {pj.x, pj.y, pj.z};
  const double c[3] = {pi.x, pi.y, pi.z};
  double dr[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double v = __dadd_rn(p[k], __dmul_rn(dn1, L[k]));
    v = __dadd_rn(v, __dmul_rn(dn2, L[3 + k]));
    v = __dadd_rn(v, __dmul_rn(dn3, L[6 + k]));
    xyz[k] = v;
    dr[k] = __dsub_rn(c[k], v);
  }
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dr[0], dr[0]), __dmul_rn(dr[1], dr[1])),
                              __dmul_rn(dr[2], dr[2])));
}

// FP32 forms of the evaluation in the binned build of large cells: relative
// vector d = (p_j - p_i) + n L with FP64 fused multiply-adds (12 FP64
// operations instead of the reference formula's ~40 with the square root),
// rounded once to FP32; the cutoff test runs on the FP32 squared length.  The
// reverse pair's vector is the exact negation, so both members of a pair
// agree.  Only where bit-identical lists are not required (fc and fc' vanish
// at the cutoff).  The unbinned builds and the MD refresh use df_rel below,
// which rounds the same way without FP64 operations.
__device__ __forceinline__ float4 fast_rel(const double4 &pi, const double4 &pj, const double *L,
                                           double dn1, double dn2, double dn3) {
  const double p[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
  float d[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) d[k] = d2f_rn(fma(dn1, L[k], fma(dn2, L[3 + k], fma(dn3, L[6 + k], p[k]))));
  return make_float4(d[0], d[1], d[2], d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

// s + e == a + b exactly (Knuth's two-sum; the _rn intrinsics keep the
// compiler from contracting or reordering it)
__device__ __forceinline__ float two_sum(float a, float b, float &e) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}

// The FP32 form's relative vector in double-float FP32 arithmetic: the
// positions and the lattice as high + low FP32 parts, the high parts summed
// exactly by two-sums, the low parts and the two-sum errors added to a low
// word, and the pair rounded once to FP32.  n L_hi is exact when every
// |n_a| <= 1 (UNIT: the cells wider than twice the cutoff); otherwise each
// product is split exactly by an FMA (p + e = n L_hi, |n| < 2^7).  It carries
// about 48 bits, so it rounds like fast_rel's FP64 vector but needs no FP64
// operation (GB300's FP64 rate is 1/74 of its FP32 rate).  Every step is odd
// under negation, so the reverse pair's vector is the exact negation.
template <bool UNIT>
__device__ __forceinline__ float4 df_rel(const float4 &pih, const float4 &pil, const float4 &pjh,
                                         const float4 &pjl, const float *Lh, const float *Ll,
                                         int n1, int n2, int n3) {
  const float f1 = (float)n1, f2 = (float)n2, f3 = (float)n3;
  const float hj[3] = {pjh.x, pjh.y, pjh.z}, hi[3] = {pih.x, pih.y, pih.z};
  const float lj[3] = {pjl.x, pjl.y, pjl.z}, li[3] = {pil.x, pil.y, pil.z};
  float d[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float e0, e1, e2, e3;
    const float p1 = __fmul_rn(f1, Lh[k]), p2 = __fmul_rn(f2, Lh[3 + k]),
                p3 = __fmul_rn(f3, Lh[6 + k]);
    float sum = two_sum(hj[k], -hi[k], e0);
    sum = two_sum(sum, p1, e1);
    sum = two_sum(sum, p2, e2);
    sum = two_sum(sum, p3, e3);
    float lo = __fsub_rn(lj[k], li[k]);
    lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(e0, e1), __fadd_rn(e2, e3)));
    if constexpr (!UNIT)  // the products' rounding errors
      lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(__fmaf_rn(f1, Lh[k], -p1), __fmaf_rn(f2, Lh[3 + k], -p2)),
                                   __fmaf_rn(f3, Lh[6 + k], -p3)));
    lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(__fmul_rn(f1, Ll[k]), __fmul_rn(f2, Ll[3 + k])),
                                 __fmul_rn(f3, Ll[6 + k])));
    d[k] = __fadd_rn(sum, lo);
  }
  return make_float4(d[0], d[1], d[2], d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

__device__ __forceinline__ void image_box(const float ext[3], const int nabc[3], const float4 &fi,
                                          const float4 &fj, int lo[3], int hi[3]) {
  const float d[3] = {fj.x - fi.x, fj.y - fi.y, fj.z - fi.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float l = ceilf(-d[a] - ext[a]), h = floorf(-d[a] + ext[a]);
    lo[a] = max(-nabc[a], (int)fmaxf(l, -1e6f));
    hi[a] = min(nabc[a], (int)fminf(h, 1e6f));
  }
}

// FP32 screen of an image: squared Cartesian length of (f_j - f_i + n) L.
// Candidates farther than rcut + margin cannot pass the exact test (the
// margin covers the FP32 rounding of the fractional coordinates).
__device__ __forceinline__ float screen_r2(const float *L32, const float fd[3], int n1, int n2,
                                           int n3) {
  const float a = fd[0] + (float)n1, b = fd[1] + (float)n2, c = fd[2] + (float)n3;
  const float x = a * L32[0] + b * L32[3] + c * L32[6];
  const float y = a * L32[1] + b * L32[4] + c * L32[7];
  const float z = a * L32[2] + b * L32[5] + c * L32[8];
  return x * x + y * y + z * z;
}

constexpr int kQueue = 256;  // survivors per warp per exact-test round

// Two kernels share this code.  WIDE: the atoms of unbinned cells wider than
// twice the cutoff on every axis (StructInfo::single), screened by their
// nearest image alone; without the general image loops the FP32 form fits
// six blocks per SM (80 registers; 0.160 -> 0.141 ms per 38 912 alloy atoms
// against one kernel at five).  !WIDE: the other unbinned cells, five blocks
// per SM (96 registers; six spill and took 0.33 ms).  Each kernel returns at
// once when the batch has no cell of its kind, and skips the others' atoms.
template <bool EXACT, bool WIDE>
__global__ void __launch_bounds__(128, (WIDE && !EXACT) ? 6 : 5)
    k_nbr_build(int N, int cap, double rcut,
                                                   const double4 *__restrict__ apos,
                                                   const float4 *__restrict__ frac32,
                                                   const float4 *__restrict__ pos2f,
                                                   const int *__restrict__ atom_struct,
                                                   const StructInfo *__restrict__ sinfo,
                                                   int *__restrict__ cnt, double4 *__restrict__ xyzr,
                                                   int *__restrict__ nj, int *__restrict__ ns,
                                                   float4 *__restrict__ d32, float *__restrict__ w32,
                                                   int *__restrict__ flags) {
  // the ring queue and, past it, one spare entry per lane for the branch-free
  // store of a lane without a survivor
  __shared__ int s_qj[kWarpsPerBlock][kQueue + 32];
  __shared__ int s_qs[kWarpsPerBlock][kQueue + 32];
  __shared__ double s_dn[2 * kMaxImage + 1];  // s_dn[n + kMaxImage] = (double)n
  if (flags[WIDE ? 4 : 3] == 0) return;  // no cell of this kernel's kind (block-uniform)
  for (int t = threadIdx.x; t < 2 * kMaxImage + 1; t += blockDim.x) s_dn[t] = (double)(t - kMaxImage);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = gw; i < N; i += nw) {
    const int sidx = atom_struct[i];
    // large cells: k_nbr_build_binned; cells of the other kind: the other kernel
    if (sinfo[sidx].nb[0] != 0 || (sinfo[sidx].single != 0) != WIDE) continue;
    const StructInfo si = sinfo[sidx];
    const double4 pi = apos[i];
    const float4 fi = frac32[i];
    // the double-float position of atom i (the FP32 form)
    float4 pih = make_float4(0.f, 0.f, 0.f, 0.f), pil = pih;
    if constexpr (!EXACT) {
      pih = pos2f[2 * (size_t)i];
      pil = pos2f[2 * (size_t)i + 1];
    }
    // FP32 screen constants of the structure (k_prep_struct): the lattice,
    // the squared bound rcut plus the fractional rounding margin, rcut^2
    const float *L32 = si.lat32;
    const float r2max = si.r2max32;
    const float rc2f = si.rc2_32;
    const float *ext = si.ext32;
    double4 *oxyz = xyzr + (size_t)i * cap;
    int *oj = nj + (size_t)i * cap;
    int *os = ns + (size_t)i * cap;
    float4 *od = d32 + (size_t)i * cap;
    float *ow = w32 + (size_t)i * cap;
    int *qj = s_qj[warp];
    int *qs = s_qs[warp];
    const unsigned lt_mask = (1u << lane) - 1u;
    int total = 0;
    int qh = 0, qt = 0;  // ring queue: candidates [qh, qt) are pending
    // exact FP64 test of queued candidates, 32 at a time (all of them when
    // `all`), hits appended in queue order = the reference order
    auto drain = [&](bool all) {
      while (qt - qh >= 32 || (all && qt > qh)) {
        // branch-free: a lane past the queue's end tests the batch's first
        // entry (queued, so in range) and reports no hit
        const int t = qh + lane;
        const bool in = t < qt;
        bool hit;
        double xyz[3] = {0, 0, 0};
        double dis = 0;
        float4 fr = make_float4(0.f, 0.f, 0.f, 0.f);
        const int e = (in ? t : qh) & (kQueue - 1);
        const int jj = qj[e], sh = qs[e];
        const int n1 = ((sh >> 16) & 255) - 128, n2 = ((sh >> 8) & 255) - 128,
                  n3 = (sh & 255) - 128;
        if (EXACT) {
          dis = ref_image(pi, apos[jj], si.lat, s_dn[n1 + kMaxImage], s_dn[n2 + kMaxImage],
                          s_dn[n3 + kMaxImage], xyz);
          hit = in & !(dis > rcut);
        } else {
          fr = df_rel<WIDE>(pih, pil, pos2f[2 * (size_t)jj], pos2f[2 * (size_t)jj + 1],
                            si.lat32, si.latl32, n1, n2, n3);
          hit = in & (fr.w <= rc2f);
        }
        __syncwarp();
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        const int q = total + __popc(m & lt_mask);
        if (hit && q < cap) {
          oj[q] = jj;
          os[q] = sh;
          if (EXACT) {
            oxyz[q] = make_double4(xyz[0], xyz[1], xyz[2], dis);
            // FP32 record for the FP32 kernels: deltaxj = xyz - pos(i)
            // (wacsf.f90:90) in FP64, rounded once to FP32
            od[q] = make_float4(d2f_rn(xyz[0] - pi.x), d2f_rn(xyz[1] - pi.y),
                                d2f_rn(xyz[2] - pi.z), d2f_rn(dis));
          } else {
            od[q] = make_float4(fr.x, fr.y, fr.z, sqrtf(fr.w));
          }
          ow[q] = frac32[jj].w;
        }
        total += __popc(m);
        qh += min(32, qt - qh);
      }
    };
    // the next chunk's fractional coordinates are loaded one chunk ahead
    float4 fj_next = lane < si.na ? frac32[si.a0 + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int base = 0; base < si.na; base += 32) {
      const int jl = base + lane;
      const bool valid = jl < si.na;
      const int j = si.a0 + jl;
      const float4 fj = fj_next;
      if (jl + 32 < si.na) fj_next = frac32[j + 32];
      const float fd[3] = {fj.x - fi.x, fj.y - fi.y, fj.z - fi.z};
      if constexpr (WIDE) {
        // the box [-d - ext, -d + ext] of each axis is narrower than 1, so it
        // holds at most one integer, the nearest to -d: n = rint(-d) is the
        // one candidate image when |d + n| <= ext on every axis and |n| <=
        // nabc - the candidates of image_box below without its bounds.  The
        // screen is screen_r2's, on the same d + n.
        float dn[3];
        int n[3];
        bool keep = valid;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float m = rintf(-fd[a]);
          dn[a] = fd[a] + m;
          n[a] = __float_as_int(m + 12582912.f) - 0x4B400000;  // m exactly, |m| < 2^22
          keep &= (fabsf(dn[a]) <= ext[a]) & (abs(n[a]) <= si.nabc[a]);
        }
        keep &= !((j == i) & (n[0] == 0) & (n[1] == 0) & (n[2] == 0));
        const float x = dn[0] * L32[0] + dn[1] * L32[3] + dn[2] * L32[6];
        const float y = dn[0] * L32[1] + dn[1] * L32[4] + dn[2] * L32[7];
        const float z = dn[0] * L32[2] + dn[1] * L32[5] + dn[2] * L32[8];
        keep &= x * x + y * y + z * z <= r2max;
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        const int e = keep ? (qt + __popc(m & lt_mask)) & (kQueue - 1) : kQueue + lane;
        qj[e] = j;
        qs[e] = ((n[0] + 128) << 16) | ((n[1] + 128) << 8) | (n[2] + 128);
        qt += __popc(m);
        __syncwarp();
        drain(false);
        continue;
      } else {
        // (branch-free: a lane past the structure's atoms has an empty box)
        int lo[3], hi[3];
        image_box(ext, si.nabc, fi, fj, lo, hi);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          lo[a] = valid ? lo[a] : 0;
          hi[a] = valid ? hi[a] : -1;
        }
        // Every lane's box holds at most one image (this chunk of j of a cell
        // narrower than twice the cutoff on some axis): one screen per lane,
        // survivors queued in lane order - the candidates and the order of the
        // general loops below, without them
        const bool none = (hi[0] < lo[0]) | (hi[1] < lo[1]) | (hi[2] < lo[2]);
        const bool one = (hi[0] == lo[0]) & (hi[1] == lo[1]) & (hi[2] == lo[2]);
        if (__all_sync(0xffffffffu, none || one)) {
          const bool self = (j == i) & (lo[0] == 0) & (lo[1] == 0) & (lo[2] == 0);
          const bool keep = one & !self & (screen_r2(L32, fd, lo[0], lo[1], lo[2]) <= r2max);
          const unsigned m = __ballot_sync(0xffffffffu, keep);
          const int e = keep ? (qt + __popc(m & lt_mask)) & (kQueue - 1) : kQueue + lane;
          qj[e] = j;
          qs[e] = ((lo[0] + 128) << 16) | ((lo[1] + 128) << 8) | (lo[2] + 128);
          qt += __popc(m);
          __syncwarp();
          drain(false);
          continue;
        }
        // FP32 screen: survivors of this lane's image box, in (n1, n2, n3) order
        int c = 0;
        if (valid)
          for (int n1 = lo[0]; n1 <= hi[0]; ++n1)
            for (int n2 = lo[1]; n2 <= hi[1]; ++n2)
              for (int n3 = lo[2]; n3 <= hi[2]; ++n3) {
                if (j == i && n1 == 0 && n2 == 0 && n3 == 0) continue;
                if (screen_r2(L32, fd, n1, n2, n3) <= r2max) ++c;
              }
        int incl = c;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, off);
          if (lane >= off) incl += t;
        }
        const int excl = incl - c;
        const int T = __shfl_sync(0xffffffffu, incl, 31);
        // survivors in canonical order (lane = j order, then shifts) enter a
        // per-warp ring queue that spans chunks; the exact FP64 test runs on
        // 32 queued candidates at a time
        for (int r0 = 0; r0 < T; r0 += kQueue - 32) {
          const int take = min(kQueue - 32, T - r0);
          if (c > 0 && excl < r0 + take && excl + c > r0) {
            int idx = excl;
            for (int n1 = lo[0]; n1 <= hi[0] && idx < r0 + take; ++n1)
              for (int n2 = lo[1]; n2 <= hi[1] && idx < r0 + take; ++n2)
                for (int n3 = lo[2]; n3 <= hi[2] && idx < r0 + take; ++n3) {
                  if (j == i && n1 == 0 && n2 == 0 && n3 == 0) continue;
                  if (screen_r2(L32, fd, n1, n2, n3) > r2max) continue;
                  if (idx >= r0) {
                    const int e = (qt + idx - r0) & (kQueue - 1);
                    qj[e] = j;
                    qs[e] = ((n1 + 128) << 16) | ((n2 + 128) << 8) | (n3 + 128);
                  }
                  ++idx;
                }
          }
          qt += take;
          __syncwarp();
          drain(false);
        }
      }  // !WIDE
    }
    drain(true);
    if (lane == 0) {
      cnt[i] = min(total, cap);
      atomicMax(flags + 1, total);
      if (total > cap) atomicOr(flags, kFlagNeighbourOverflow);
    }
  }
}

// Neighbour list of an atom of a binned cell: candidates from the 27 bins
// around its own, the same FP32 screen and exact FP64 test as k_nbr_build,
// hits collected in shared memory and sorted by (j, n1, n2, n3) - the
// reference's order - before they are written, so the list is identical to
// the O(na) scan's.  The image of candidate j is n = s - m_j + m_i, with s the
// bin-wrap shift and m the atoms' own wrap shifts.
template <bool EXACT>
__global__ void __launch_bounds__(128) k_nbr_build_binned(
    int N, int cap, int hit_cap, double rcut, const double4 *__restrict__ apos,
    const float4 *__restrict__ frac32, const int *__restrict__ atom_struct,
    const StructInfo *__restrict__ sinfo, const int *__restrict__ bin_start,
    const int *__restrict__ bin_atoms, const int *__restrict__ atom_bin,
    const int *__restrict__ atom_m, int *__restrict__ cnt, double4 *__restrict__ xyzr,
    int *__restrict__ nj, int *__restrict__ ns, float4 *__restrict__ d32, float *__restrict__ w32,
    int *__restrict__ flags) {
  extern __shared__ __align__(16) unsigned char smb[];
  __shared__ double s_dn[2 * kMaxImage + 1];
  for (int t = threadIdx.x; t < 2 * kMaxImage + 1; t += blockDim.x) s_dn[t] = (double)(t - kMaxImage);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // per warp: hit_cap keys (8 B), records (32 B)
  unsigned long long *keys =
      reinterpret_cast<unsigned long long *>(smb) + (size_t)warp * hit_cap;
  double4 *recs = reinterpret_cast<double4 *>(smb + (size_t)kWarpsPerBlock * hit_cap * 8) +
                  (size_t)warp * hit_cap;
  int *order = reinterpret_cast<int *>(smb + (size_t)kWarpsPerBlock * hit_cap * 40) +
               (size_t)warp * hit_cap;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = gw; i < N; i += nw) {
    const StructInfo si = sinfo[atom_struct[i]];
    if (si.nb[0] == 0) continue;
    const double4 pi = apos[i];
    const float4 fi = frac32[i];
    const float *L32 = si.lat32;  // FP32 screen constants (k_prep_struct)
    const float r2max = si.r2max32;
    const float rc2f = si.rc2_32;
    const int mi = atom_m[i];
    const int mi3[3] = {((mi >> 16) & 255) - 128, ((mi >> 8) & 255) - 128, (mi & 255) - 128};
    const int local = atom_bin[i] - si.bin0;
    const int bi[3] = {local / (si.nb[1] * si.nb[2]), (local / si.nb[2]) % si.nb[1],
                       local % si.nb[2]};
    int total = 0;
    for (int d = 0; d < 27; ++d) {
      int c[3], sh[3];
      const int dd[3] = {d / 9 - 1, (d / 3) % 3 - 1, d % 3 - 1};
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        c[a] = bi[a] + dd[a];
        sh[a] = c[a] < 0 ? -1 : (c[a] >= si.nb[a] ? 1 : 0);
        c[a] -= sh[a] * si.nb[a];
      }
      const int gid = si.bin0 + (c[0] * si.nb[1] + c[1]) * si.nb[2] + c[2];
      const int b0 = bin_start[gid], b1 = bin_start[gid + 1];
      for (int t0 = b0; t0 < b1; t0 += 32) {
        const int t = t0 + lane;
        bool hit = false;
        unsigned long long key = 0;
        double4 rec = make_double4(0, 0, 0, 0);
        if (t < b1) {
          const int j = bin_atoms[t];
          const int mj = atom_m[j];
          const int n1 = sh[0] - (((mj >> 16) & 255) - 128) + mi3[0];
          const int n2 = sh[1] - (((mj >> 8) & 255) - 128) + mi3[1];
          const int n3 = sh[2] - ((mj & 255) - 128) + mi3[2];
          const bool self = j == i && n1 == 0 && n2 == 0 && n3 == 0;
          const bool inrange = n1 >= -kMaxImage && n1 <= kMaxImage && n2 >= -kMaxImage &&
                               n2 <= kMaxImage && n3 >= -kMaxImage && n3 <= kMaxImage;
          if (!self && inrange) {
            const float4 fj = frac32[j];
            const float fd[3] = {fj.x - fi.x, fj.y - fi.y, fj.z - fi.z};
            if (screen_r2(L32, fd, n1, n2, n3) <= r2max) {
              if (EXACT) {
                double xyz[3];
                const double dis = ref_image(pi, apos[j], si.lat, s_dn[n1 + kMaxImage],
                                             s_dn[n2 + kMaxImage], s_dn[n3 + kMaxImage], xyz);
                hit = !(dis > rcut);
                rec = make_double4(xyz[0], xyz[1], xyz[2], dis);
              } else {
                const float4 fr = fast_rel(pi, apos[j], si.lat, s_dn[n1 + kMaxImage],
                                           s_dn[n2 + kMaxImage], s_dn[n3 + kMaxImage]);
                hit = fr.w <= rc2f;
                *reinterpret_cast<float4 *>(&rec) = fr;  // FP32 record in the slot's bytes
              }
              key = ((unsigned long long)j << 24) |
                    (unsigned long long)(((n1 + 128) << 16) | ((n2 + 128) << 8) | (n3 + 128));
            }
          }
        }
        const unsigned mball = __ballot_sync(0xffffffffu, hit);
        const int q = total + __popc(mball & lt_mask);
        if (hit && q < hit_cap) {
          keys[q] = key;
          recs[q] = rec;
        }
        total += __popc(mball);
      }
    }
    __syncwarp();
    const int nh = min(total, hit_cap);
    // bitonic sort of the hit keys (with their positions) in shared memory
    int n2p = 1;
    while (n2p < nh) n2p <<= 1;
    for (int t = lane; t < n2p; t += 32) {
      order[t] = t;
      if (t >= nh) keys[t] = ~0ull;
    }
    __syncwarp();
    for (int k = 2; k <= n2p; k <<= 1)
      for (int jj = k >> 1; jj > 0; jj >>= 1) {
        for (int t = lane; t < n2p; t += 32) {
          const int p = t ^ jj;
          if (p > t) {
            const bool up = (t & k) == 0;
            const unsigned long long a = keys[t], b = keys[p];
            if ((a > b) == up) {
              keys[t] = b;
              keys[p] = a;
              const int o = order[t];
              order[t] = order[p];
              order[p] = o;
            }
          }
        }
        __syncwarp();
      }
    const int nout = min(total, min(cap, hit_cap));
    double4 *oxyz = xyzr + (size_t)i * cap;
    for (int q = lane; q < nout; q += 32) {
      const unsigned long long key = keys[q];
      const double4 rec = recs[order[q]];
      const int j = (int)(key >> 24);
      nj[(size_t)i * cap + q] = j;
      ns[(size_t)i * cap + q] = (int)(key & 0xFFFFFFull);
      if (EXACT) {
        oxyz[q] = rec;
        d32[(size_t)i * cap + q] = make_float4(d2f_rn(rec.x - pi.x), d2f_rn(rec.y - pi.y),
                                               d2f_rn(rec.z - pi.z), d2f_rn(rec.w));
      } else {
        const float4 fr = *reinterpret_cast<const float4 *>(&rec);
        d32[(size_t)i * cap + q] = make_float4(fr.x, fr.y, fr.z, sqrtf(fr.w));
      }
      w32[(size_t)i * cap + q] = frac32[j].w;
    }
    if (lane == 0) {
      cnt[i] = nout;
      atomicMax(flags + 1, total);
      if (total > cap || total > hit_cap) atomicOr(flags, kFlagNeighbourOverflow);
    }
    __syncwarp();
  }
}

// Reverse slot of every (i, q): the slot of (partner -> i, -shift) in the
// partner's list, found by binary search over its (j, shift) ordered keys.
__global__ void k_nbr_reverse(int N, int cap, const int *__restrict__ cnt,
                              const int *__restrict__ nj, const int *__restrict__ ns,
                              int *__restrict__ rev, int *__restrict__ orphans, int orphan_cap,
                              int *__restrict__ flags) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = gw; i < N; i += nw) {
    const int P = cnt[i];
    for (int q = lane; q < P; q += 32) {
      const size_t idx = (size_t)i * cap + q;
      const int j = nj[idx];
      const int s = ns[idx];
      const int n1 = ((s >> 16) & 255) - 128, n2 = ((s >> 8) & 255) - 128, n3 = (s & 255) - 128;
      const int want = ((128 - n1) << 16) | ((128 - n2) << 8) | (128 - n3);
      const int *kj = nj + (size_t)j * cap;
      const int *ks = ns + (size_t)j * cap;
      int lo = 0, hi = cnt[j];
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        int a = kj[mid];
        bool less = (a < i) || (a == i && ks[mid] < want);
        if (less) lo = mid + 1; else hi = mid;
      }
      int r = -1;
      if (lo < cnt[j] && kj[lo] == i && ks[lo] == want) r = lo;
      rev[idx] = r;
      if (r < 0) {
        int o = atomicAdd(flags + 2, 1);
        if (o < orphan_cap) orphans[o] = (int)idx;
        else atomicOr(flags, kFlagOrphanOverflow);
      }
    }
  }
}

// Verlet-list refresh: the slots of a list built with a larger cutoff keep
// their (partner, image shift); their image positions, distances and FP32
// records are recomputed from the current positions with the build's exact
// formula.  Slots now beyond an SF cutoff contribute exactly zero in every
// descriptor kernel, so the result equals a fresh build's up to summation
// order.  One thread per slot.
template <bool EXACT>
__global__ void k_nbr_refresh(int N, int cap, const int *__restrict__ cnt,
                              const int *__restrict__ nj, const int *__restrict__ ns,
                              const double4 *__restrict__ apos, const float4 *__restrict__ pos2f,
                              const int *__restrict__ atom_struct,
                              const StructInfo *__restrict__ sinfo, double4 *__restrict__ xyzr,
                              float4 *__restrict__ d32) {
  __shared__ double s_dn[2 * kMaxImage + 1];
  for (int t = threadIdx.x; t < 2 * kMaxImage + 1; t += blockDim.x) s_dn[t] = (double)(t - kMaxImage);
  __syncthreads();
  const size_t total = (size_t)N * cap;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx / cap), q = (int)(idx - (size_t)i * cap);
    if (q >= cnt[i]) continue;
    const int j = nj[idx], sh = ns[idx];
    const int n1 = ((sh >> 16) & 255) - 128, n2 = ((sh >> 8) & 255) - 128, n3 = (sh & 255) - 128;
    const double4 pi = apos[i];
    const double *L = sinfo[atom_struct[i]].lat;
    if (EXACT) {
      double xyz[3];
      const double dis = ref_image(pi, apos[j], L, s_dn[n1 + kMaxImage], s_dn[n2 + kMaxImage],
                                   s_dn[n3 + kMaxImage], xyz);
      xyzr[idx] = make_double4(xyz[0], xyz[1], xyz[2], dis);
      d32[idx] = make_float4(d2f_rn(xyz[0] - pi.x), d2f_rn(xyz[1] - pi.y),
                             d2f_rn(xyz[2] - pi.z), d2f_rn(dis));
    } else {
      // double-float, as the wide build kernel: no FP64 operation per slot
      const StructInfo &si = sinfo[atom_struct[i]];
      const float4 fr = df_rel<false>(pos2f[2 * (size_t)i], pos2f[2 * (size_t)i + 1],
                                      pos2f[2 * (size_t)j], pos2f[2 * (size_t)j + 1], si.lat32,
                                      si.latl32, n1, n2, n3);
      d32[idx] = make_float4(fr.x, fr.y, fr.z, sqrtf(fr.w));
    }
  }
}

// FGET_BOND (gappy/libgap/get_bond.f90:47-78): minimum over all kept images.
__global__ void __launch_bounds__(128) k_min_bond(int N, double rcut,
                                                  const double4 *__restrict__ apos,
                                                  const float4 *__restrict__ frac32,
                                                  const int *__restrict__ atom_struct,
                                                  const StructInfo *__restrict__ sinfo,
                                                  unsigned long long *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = gw; i < N; i += nw) {
    const StructInfo si = sinfo[atom_struct[i]];
    const double4 pi = apos[i];
    const float4 fi = frac32[i];
    const float ext[3] = {(float)si.ext[0], (float)si.ext[1], (float)si.ext[2]};
    double best = 10.0;  // get_bond.f90:38
    for (int jl = lane; jl < si.na; jl += 32) {
      const int j = si.a0 + jl;
      const double4 pj = apos[j];
      int lo[3], hi[3];
      image_box(ext, si.nabc, fi, frac32[j], lo, hi);
      for (int n1 = lo[0]; n1 <= hi[0]; ++n1)
        for (int n2 = lo[1]; n2 <= hi[1]; ++n2)
          for (int n3 = lo[2]; n3 <= hi[2]; ++n3) {
            if (j == i && n1 == 0 && n2 == 0 && n3 == 0) continue;
            double xyz[3];
            double dis = ref_image(pi, pj, si.lat, (double)n1, (double)n2, (double)n3, xyz);
            if (dis > rcut) continue;
            if (dis < best) best = dis;
          }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, off));
    if (lane == 0) atomicMin(out, (unsigned long long)__double_as_longlong(best));
  }
}

int grid_for_warps(int nwarps_needed) {
  const int sms = device_sms();
  int blocks = (nwarps_needed + kWarpsPerBlock - 1) / kWarpsPerBlock;
  int maxb = sms * 16;
  return blocks < maxb ? (blocks > 0 ? blocks : 1) : maxb;
}

}  // namespace

void launch_prep(const gapgb_model *m, Workspace &ws, int S, int N, const int *d_atom_off,
                 const int *d_species, const double *d_lat, const double *d_pos, double rcut,
                 cudaStream_t st, bool allow_bins) {
  k_prep_struct<<<(S + 127) / 128, 128, 0, st>>>(S, d_atom_off, d_lat, rcut, allow_bins ? 1 : 0,
                                                 ws.sinfo, ws.d_flags);
  k_prep_atoms<<<(N + 255) / 256, 256, 0, st>>>(N, S, d_atom_off, d_species, d_pos, m->d_sf,
                                                 ws.sinfo, ws.atom_struct, ws.apos, ws.frac32,
                                                 ws.pos2f, ws.d_flags);
}

void launch_neighbors(Workspace &ws, int S, int N, int max_atoms, int cap, double rcut,
                      cudaStream_t st, bool exact) {
  auto build_wide = exact ? k_nbr_build<true, true> : k_nbr_build<false, true>;
  auto build = exact ? k_nbr_build<true, false> : k_nbr_build<false, false>;
  auto build_binned = exact ? k_nbr_build_binned<true> : k_nbr_build_binned<false>;
  // cells wider than twice the cutoff, then the other unbinned cells
  for (auto fn : {build_wide, build})
    fn<<<grid_for_warps(N), 32 * kWarpsPerBlock, 0, st>>>(
        N, cap, rcut, ws.apos, ws.frac32, ws.pos2f, ws.atom_struct, ws.sinfo, ws.nbr_cnt,
        ws.nbr_xyz, ws.nbr_j, ws.nbr_s, ws.nbr_d32, ws.nbr_w32, ws.d_flags);
  if (max_atoms < kBinMinAtoms) return;  // no structure was binned (launch_prep)
  int *total = ws.bin_count + N;  // last entry of the count array holds the bin total
  cudaMemsetAsync(ws.bin_count, 0, sizeof(int) * (size_t)(N + 1), st);
  k_bin_offsets<<<1, 32, 0, st>>>(S, ws.sinfo, total);
  k_bin_count<<<(N + 255) / 256, 256, 0, st>>>(N, ws.frac32, ws.atom_struct, ws.sinfo,
                                               ws.bin_count, ws.atom_bin, ws.atom_slot,
                                               ws.atom_m);
  k_bin_scan<<<1, 1024, 0, st>>>(total, ws.bin_count, ws.bin_start);
  k_bin_fill<<<(N + 255) / 256, 256, 0, st>>>(N, ws.atom_struct, ws.sinfo, ws.atom_bin,
                                              ws.atom_slot, ws.bin_start, ws.bin_atoms);
  // hits beyond the capacity are counted (overflow) but not stored; the
  // per-warp sort buffer is a power of two (the bitonic network's size)
  int hit_cap = 32;
  while (hit_cap < cap && hit_cap < 1024) hit_cap <<= 1;
  const size_t smem = (size_t)kWarpsPerBlock * hit_cap * (8 + 32 + 4);
  kernel_smem((const void *)build_binned, (int)smem);
  build_binned<<<grid_for_warps(N), 32 * kWarpsPerBlock, smem, st>>>(
      N, cap, hit_cap, rcut, ws.apos, ws.frac32, ws.atom_struct, ws.sinfo, ws.bin_start,
      ws.bin_atoms, ws.atom_bin, ws.atom_m, ws.nbr_cnt, ws.nbr_xyz, ws.nbr_j, ws.nbr_s,
      ws.nbr_d32, ws.nbr_w32, ws.d_flags);
}

void launch_refresh(Workspace &ws, int N, int cap, cudaStream_t st, bool exact) {
  const int sms = device_sms();
  const size_t total = (size_t)N * cap;
  const size_t want = (total + 255) / 256;
  const int grid = (int)std::min<size_t>(want > 0 ? want : 1, (size_t)sms * 8);
  auto fn = exact ? k_nbr_refresh<true> : k_nbr_refresh<false>;
  fn<<<grid, 256, 0, st>>>(N, cap, ws.nbr_cnt, ws.nbr_j, ws.nbr_s, ws.apos, ws.pos2f,
                           ws.atom_struct, ws.sinfo, ws.nbr_xyz, ws.nbr_d32);
}

void launch_reverse(Workspace &ws, int N, int cap, cudaStream_t st) {
  k_nbr_reverse<<<grid_for_warps(N), 32 * kWarpsPerBlock, 0, st>>>(
      N, cap, ws.nbr_cnt, ws.nbr_j, ws.nbr_s, ws.nbr_rev, ws.orphans, ws.orphan_cap, ws.d_flags);
}

void launch_min_bond(Workspace &ws, int N, double rcut, double *d_out, cudaStream_t st) {
  k_min_bond<<<grid_for_warps(N), 32 * kWarpsPerBlock, 0, st>>>(
      N, rcut, ws.apos, ws.frac32, ws.atom_struct, ws.sinfo, (unsigned long long *)d_out);
}

}  // namespace gapgb
