// gapgb_internal.h - shared definitions of the GB300 CALYPSO-GAP evaluator.
//
// Device data layout (one packed ragged batch of S structures, N atoms):
//   apos[N]          double4 {x, y, z, species weight}
//   atom_struct[N]   structure index of each atom
//   sinfo[S]         per-structure lattice, inverse lattice, image counts
//   nbr_cnt[N]       neighbours of atom i (<= cap)
//   nbr_xyz[N*cap]   double4 {image x, y, z, r} - the reference's
//                    neighbor(i,q,1:4) (gappy/libgap/gap_calc.f90:112-113)
//   nbr_j[N*cap]     partner atom (global index)
//   nbr_s[N*cap]     packed image shift ((n1+128)<<16 | (n2+128)<<8 | n3+128)
//   nbr_rev[N*cap]   slot of the reverse pair in the partner's list, -1 if absent
//   G[N*D]           descriptors (T = double or float), the reference's XX^T
//   e[N]             atomic energies (double)
//   dedg[N*D]        dE/dG (T)
//   gslot[N*cap]     Vec4<T> {sum_d dedg_d dG_d/dp_q, 0}: gradient of atom i's
//                    energy with respect to the position of neighbour slot q
//   wvir[N*9]        per-atom virial sum_q (p_q - r_i)_a gslot_q,b (double)
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gapgb.h"

namespace gapgb {

constexpr double kPiRef = 3.141592654;        // gap_calc.f90:59, wacsf.f90:31
constexpr double kGPa2eVPang = 6.24219e-3;    // gap_calc.f90:9
constexpr int kMaxSF = 128;                   // symmetry functions per model
constexpr int kMaxRC = 16;                    // distinct SF cutoffs
constexpr int kMaxAlpha = 16;                 // distinct angular exponents
constexpr int kMaxImage = 127;                // |n_a| limit of the packed shift
constexpr int kWarpsPerBlock = 4;
constexpr int kMaxSpecies = 128;

// Device error flags (bit positions in Workspace::d_flags[0]).
enum : int {
  kFlagNeighbourOverflow = 1,
  kFlagUnknownSpecies = 2,
  kFlagImageLimit = 4,
  kFlagOrphanOverflow = 8,
  kFlagTimeout = 16,
  kFlagSkinExceeded = 32,  // MD: an atom moved more than half the skin since the last rebuild
  kFlagNotPositiveDefinite = 64,  // fit: a Cholesky pivot was not positive
  kFlagForceRange = 128,  // FP32 gradient: a slot-gradient term beyond the fixed-point range
};

// Symmetry-function table as the kernels read it.  Angular SFs are grouped by
// distinct cutoff (rc) so that fc(r_jk) is evaluated once per triplet and
// cutoff; per-slot fc and exp(-alpha r^2) tables live in shared memory.
struct SFDev {
  int nsf;       // D = 2*nsf descriptor entries are written (wacsf.f90:86-87)
  int D;         // descriptor length of the model (>= 2*nsf)
  int nrad, nang;
  int nrc;       // distinct cutoffs over all SFs
  int nalpha;    // distinct angular alphas
  double max_ang_rc, max_rc;
  double rc_val[kMaxRC];
  double alpha_val[kMaxAlpha];
  // radial SFs (types 1 and 3)
  int rad_d[kMaxSF];
  int rad_rc[kMaxSF];
  double rad_alpha[kMaxSF];  // type 1: alpha; type 3: 4.0 (wacsf.f90:439)
  double rad_rs[kMaxSF];     // type 1: 0;     type 3: R_s (wacsf.f90:438)
  // angular SFs (types 2 and 4) sorted by cutoff index
  int ang_d[kMaxSF];
  int ang_rc[kMaxSF];
  int ang_alpha[kMaxSF];
  int ang_izeta[kMaxSF];     // zeta if a small positive integer, else -1
  double ang_lambda[kMaxSF]; // +1 (type 2), -1 (type 4)
  double ang_zeta[kMaxSF];
  double ang_pref[kMaxSF];   // 2^(1-zeta)
  // angular SFs of cutoff group g are ang_grp_start[g] .. ang_grp_start[g+1]-1
  int n_ang_grp;
  int ang_grp_rc[kMaxRC];
  int ang_grp_start[kMaxRC + 1];
  // species weights (gap_calc.f90:75-83; the last matching entry wins)
  int nspecies;
  int species_z[kMaxSpecies];
  double species_w[kMaxSpecies];
};

// The SF table in the arithmetic type of a descriptor kernel (no FP64 in the
// FP32 kernels' loops).  Radial and angular entries as in SFDev; angular
// entries sorted by cutoff group.
constexpr int kAngChunk = 16;  // angular SFs accumulated in registers per pass
template <typename T>
struct SFT {
  int nsf, D, nrad, nang, nrc, nalpha, n_ang_grp;
  T max_ang_rc;
  T rc_val[kMaxRC];
  T pi_over_rc[kMaxRC];
  T alpha_val[kMaxAlpha];
  int rad_d[kMaxSF];
  int rad_rc[kMaxSF];
  T rad_alpha[kMaxSF];
  T rad_rs[kMaxSF];
  int ang_d[kMaxSF];
  // rc | alpha << 8 | izeta << 16 | (lambda < 0) << 24 (izeta 0: non-integer zeta)
  int ang_code[kMaxSF];
  T ang_lambda[kMaxSF];
  T ang_zeta[kMaxSF];
  T ang_pref[kMaxSF];
  int ang_grp_rc[kMaxRC];
  int ang_grp_start[kMaxRC + 1];
  // grouped form of the angular SFs: SF s = (alpha index q_s, combination c_s
  // of lambda and integer zeta).  fast_nal / fast_nc are the padded grid sizes
  // of the templated fast kernels (0 when the model does not qualify: more
  // than one angular cutoff, more than 4 alphas, more than 8 combinations or
  // a non-integer zeta).
  int ncomb;
  int comb_iz[8];
  T comb_lam[8];
  int ang_comb[kMaxSF];
  int fast_nal, fast_nc;
  // 1 when the combinations are exactly zeta {1, 2, 4} x lambda {+1, -1},
  // renumbered c = 2 log2(zeta) + (lambda < 0): the powers then have a
  // closed form (fast kernels' STD variant)
  int std6;
};

template <typename T>
inline SFT<T> make_sft(const SFDev &s) {
  SFT<T> t{};
  t.nsf = s.nsf;
  t.D = s.D;
  t.nrad = s.nrad;
  t.nang = s.nang;
  t.nrc = s.nrc;
  t.nalpha = s.nalpha;
  t.n_ang_grp = s.n_ang_grp;
  t.max_ang_rc = (T)s.max_ang_rc;
  for (int q = 0; q < s.nrc; ++q) {
    t.rc_val[q] = (T)s.rc_val[q];
    t.pi_over_rc[q] = (T)(kPiRef / s.rc_val[q]);
  }
  for (int q = 0; q < s.nalpha; ++q) t.alpha_val[q] = (T)s.alpha_val[q];
  for (int q = 0; q < s.nrad; ++q) {
    t.rad_d[q] = s.rad_d[q];
    t.rad_rc[q] = s.rad_rc[q];
    t.rad_alpha[q] = (T)s.rad_alpha[q];
    t.rad_rs[q] = (T)s.rad_rs[q];
  }
  for (int q = 0; q < s.nang; ++q) {
    t.ang_d[q] = s.ang_d[q];
    const int iz = s.ang_izeta[q] > 0 ? s.ang_izeta[q] : 0;
    t.ang_code[q] = s.ang_rc[q] | (s.ang_alpha[q] << 8) | (iz << 16) |
                    (s.ang_lambda[q] < 0 ? (1 << 24) : 0);
    t.ang_lambda[q] = (T)s.ang_lambda[q];
    t.ang_zeta[q] = (T)s.ang_zeta[q];
    t.ang_pref[q] = (T)s.ang_pref[q];
  }
  for (int g = 0; g < s.n_ang_grp; ++g) t.ang_grp_rc[g] = s.ang_grp_rc[g];
  for (int g = 0; g <= s.n_ang_grp; ++g) t.ang_grp_start[g] = s.ang_grp_start[g];
  // combinations of (lambda, integer zeta)
  bool ok = s.n_ang_grp <= 1 && s.nalpha <= 4;
  t.ncomb = 0;
  for (int q = 0; q < s.nang && ok; ++q) {
    if (s.ang_izeta[q] <= 0) { ok = false; break; }
    int c = -1;
    for (int k = 0; k < t.ncomb; ++k)
      if (t.comb_iz[k] == s.ang_izeta[q] && t.comb_lam[k] == (T)s.ang_lambda[q]) c = k;
    if (c < 0) {
      if (t.ncomb == 8) { ok = false; break; }
      c = t.ncomb++;
      t.comb_iz[c] = s.ang_izeta[q];
      t.comb_lam[c] = (T)s.ang_lambda[q];
    }
    t.ang_comb[q] = c;
  }
  t.fast_nal = t.fast_nc = 0;
  t.std6 = 0;
  if (ok && t.ncomb == 6) {
    bool seen[6] = {false, false, false, false, false, false};
    bool std = true;
    for (int c = 0; c < 6 && std; ++c) {
      const int iz = t.comb_iz[c];
      const int lg = iz == 1 ? 0 : (iz == 2 ? 1 : (iz == 4 ? 2 : -1));
      if (lg < 0) { std = false; break; }
      const int k = 2 * lg + (t.comb_lam[c] < (T)0 ? 1 : 0);
      if (seen[k]) std = false;
      seen[k] = true;
    }
    if (std) {
      int remap[8];
      for (int c = 0; c < 6; ++c) {
        const int iz = t.comb_iz[c];
        remap[c] = 2 * (iz == 1 ? 0 : (iz == 2 ? 1 : 2)) + (t.comb_lam[c] < (T)0 ? 1 : 0);
      }
      for (int q = 0; q < s.nang; ++q) t.ang_comb[q] = remap[t.ang_comb[q]];
      for (int k = 0; k < 6; ++k) {
        t.comb_iz[k] = 1 << (k / 2);
        t.comb_lam[k] = (k & 1) ? (T)-1 : (T)1;
      }
      t.std6 = 1;
    }
  }
  if (ok) {
    const int na = s.nalpha < 1 ? 1 : s.nalpha;
    t.fast_nal = na <= 1 ? 1 : (na <= 2 ? 2 : 4);
    const int nc = t.ncomb < 1 ? 1 : t.ncomb;
    t.fast_nc = nc <= 2 ? 2 : (nc <= 4 ? 4 : (nc <= 6 ? 6 : 8));
    for (int c = t.ncomb; c < 8; ++c) {  // padding combinations carry zero weight
      t.comb_iz[c] = 1;
      t.comb_lam[c] = (T)1;
    }
  }
  return t;
}

struct StructInfo {
  double lat[9];   // rows = lattice vectors
  double linv[9];  // inverse: fractional f = d * linv (row vector)
  double ext[3];   // conservative |f_a + n_a| bound: rcut * |column a of linv|
  double volume;   // |det(lat)| (gap_calc.f90:201)
  // FP32 forms of the screen's constants, formed once per structure (the
  // conversions run on the narrow FP64 pipe): the lattice, ext, the squared
  // screen bound (rcut plus the fractional rounding margin) and rcut^2
  float lat32[9];
  float latl32[9];  // lat - lat32, rounded to FP32: the lattice as a double-float pair
  float ext32[3];
  float r2max32, rc2_32;
  int nabc[3];     // gap_calc.f90:85-88
  int a0, na;
  // spatial bins of a large cell (nb[0] == 0: not binned): nb[a] bins of
  // fractional width >= ext[a] per axis, global bin ids bin0 .. bin0 + nb0 nb1 nb2 - 1
  int nb[3];
  int bin0;
  // 1 when 2 ext[a] < 1 on every axis (a cell wider than twice the cutoff):
  // then at most one image of an atom, the nearest, can lie within the cutoff
  int single;
};

constexpr int kPairCap = 1024;  // recorded angular pairs per atom
constexpr int kBinMinAtoms = 2048;  // cells smaller than this use the O(na) scan

template <typename T> struct Vec4;
template <> struct Vec4<double> { using type = double4; };
template <> struct Vec4<float> { using type = float4; };

struct HostModel {
  int nspecies = 0;
  std::vector<int> species_z;
  std::vector<double> species_w;
  int nsf = 0;
  std::vector<int> sf_type;
  std::vector<double> sf_alpha, sf_cutoff, sf_zeta;
  int M = 0, D = 0;
  std::vector<double> theta, mm, coeff;
  double rcut = 6.0;
};

struct Workspace {
  int N = 0, S = 0, cap = 0, D = 0;
  size_t bytes = 0;
  // inputs (host-buffer path copies here)
  int *d_atom_off = nullptr, *d_species = nullptr;
  double *d_lat = nullptr, *d_pos = nullptr;
  // outputs (host-buffer path)
  double *d_energy = nullptr, *d_force = nullptr, *d_stress = nullptr, *d_atom_e = nullptr;
  // internal
  double4 *apos = nullptr;
  float4 *frac32 = nullptr;   // fractional coordinates (FP32) for image pruning
  float4 *pos2f = nullptr;    // each position as FP32 high [2 i] and low [2 i + 1] parts
                              // (the FP32 neighbour form's relative vectors)
  int *atom_struct = nullptr;
  StructInfo *sinfo = nullptr;
  int *nbr_cnt = nullptr, *nbr_j = nullptr, *nbr_s = nullptr, *nbr_rev = nullptr;
  double4 *nbr_xyz = nullptr;
  float4 *nbr_d32 = nullptr;  // FP32 {p_q - r_i, r} of every slot (FP32 kernels)
  float *nbr_w32 = nullptr;   // FP32 weight of every slot's atom
  void *G = nullptr, *dedg = nullptr, *gslot = nullptr;
  double *e = nullptr, *wvir = nullptr;
  double *red_part = nullptr;  // per-structure partial sums [S][64][7]
  // spatial bins of large cells (neighbour build)
  int *bin_count = nullptr, *bin_start = nullptr, *bin_atoms = nullptr;
  int *atom_bin = nullptr, *atom_slot = nullptr, *atom_m = nullptr;
  int *d_flags = nullptr;     // [0] error bits, [1] max neighbour count, [2] orphan count,
                              // [3] / [4] nonzero when the batch has unbinned cells that are
                              // not / are wider than twice the cutoff (k_prep_struct)
  int *orphans = nullptr;     // orphan slot list
  int orphan_cap = 0;
  int *h_flags = nullptr;     // pinned mirror of d_flags
  void *gpr_scratch = nullptr;  // split-K partial sums of the GPR
  size_t gpr_scratch_size = 0;
  void *tc_scratch = nullptr;   // atom operand tiles of the tensor-core GPR
  size_t tc_scratch_size = 0;
  // contributing angular pairs (j | k << 8) of every atom, recorded by the
  // grouped FP32 descriptor kernel and streamed by its gradient kernel
  unsigned short *pairs = nullptr;  // [N][kPairCap]
  int *pair_cnt = nullptr;      // [N] pairs found (may exceed kPairCap: then re-enumerated)
};

// GPR predictive variance (variance.cu): the caller's qmm and its device forms
struct VarState {
  std::vector<double> qmm;            // [M][M] row-major; empty = none attached
  double *d_q64 = nullptr;            // [Mp][Mp] FP64, zero-padded (FP64 form)
  unsigned char *d_qimg = nullptr;    // split-BF16 operand tiles (tensor-core form)
  double *d_mu64 = nullptr;           // [D] mean of mm / theta (tensor-core form)
  float *d_mc32 = nullptr;            // [M][D] mm / theta - mu (tensor-core form)
  void *kbuf = nullptr;               // K of one chunk of atoms (FP64 rows or tiles)
  void *part = nullptr;               // per-row partial dots [rows][column tiles]
  void *covf = nullptr;               // [N] covf of the last call (FP64)
  void *var = nullptr;                // [S] VARIANCE of the last call (FP64)
  void *xc = nullptr;                 // centred FP32 descriptors of one chunk
  size_t kbuf_bytes = 0, part_bytes = 0, covf_bytes = 0, var_bytes = 0, xc_bytes = 0;
};

}  // namespace gapgb

struct gapgb_model {
  gapgb::HostModel host;
  gapgb::SFDev sfh;                    // host copy of the SF table
  gapgb::SFDev *d_sf = nullptr;
  gapgb::SFT<double> *d_sft64 = nullptr;
  gapgb::SFT<float> *d_sft32 = nullptr;
  gapgb::SFT<float> sft32h{};          // host copy (kernel selection)
  double *d_mmt = nullptr;             // M x D, mm / theta (FP64)
  float *d_mmt32 = nullptr;            // M x D, mm / theta (FP32)
  double *d_invth = nullptr;           // D, 1 / theta
  float *d_invth32 = nullptr;
  double *d_coeff = nullptr;           // M
  float *d_coeff32 = nullptr;
  void *d_tc = nullptr;                // tensor-core operand images (gpr_tc.cu)
  size_t tc_bytes = 0;
  int tc_tiles = 0;
  void *d_tf32 = nullptr;              // TF32 operand images (gpr_tf32.cu)
  size_t tf32_bytes = 0;
  int tf32_tiles = 0;
  int device = 0;
  int precision = GAPGB_PREC_FP64;
  int cap = 256;
  int caps_hint = 0;                   // slot count the host-buffer calls size the descriptor kernels for
  bool generic_kernels = false;        // force the generic FP32 descriptor kernels
  cudaStream_t stream = nullptr;       // internal stream of the host-buffer calls
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int pipelines = 2;                   // GAPGB_OPT_PIPELINES
  cudaStream_t side = nullptr;         // second pipeline's stream
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;  // no timing
  bool profile_stages = false;
  float stage_ms[4] = {0, 0, 0, 0};
  gapgb::Workspace ws;
  // learned surrogate (not owned) and its fallback buffers
  gapgb_surrogate *surrogate = nullptr;
  double surr_threshold = 0.005;
  double surr_contact = 0.0;   // Angstrom: a neighbour closer than this forces the GPR
  double surr_gspread = 0.0;   // eV per descriptor unit: a dE/dG spread above this forces it
  int surr_cap = 0;
  float *surr_std = nullptr;   // committee std per atom (eV)
  float *surr_gstd = nullptr;  // members' dE/dG spread per atom (eV per descriptor unit)
  int *fb_rows = nullptr;      // atoms that take the GPR
  int *fb_count = nullptr;
  void *fb_scratch = nullptr;  // partial sums of the fallback GPR
  gapgb::VarState var;         // predictive variance (gapgb_model_set_qmm)
  float var_ms = 0.f;          // device time of the last variance kernels (profiling)
  // CUDA graphs (gapgb_graph, gapgb_md) that captured this model's buffers:
  // while any is alive, nothing they captured may move.  Shared, so a graph
  // freed after its model still decrements valid memory.
  std::shared_ptr<std::atomic<int>> live_graphs = std::make_shared<std::atomic<int>>(0);
};

namespace gapgb {

// fit.cu
gapgb_status fit_enqueue(gapgb_model *m, int S, int N, int cap, int capS, const int *d_off,
                         const double *d_G, const double *energy, const double *forces,
                         const double *stress, double sigma_e, double sigma_f, double sigma_s,
                         double jitter, double *coeff, cudaStream_t st);

// launch_cache.cpp: launch attributes set / queried once per device
// (a larger shared-memory size raises the limit; the limit never shrinks)
void kernel_smem(const void *fn, int bytes, bool max_carveout = false);
// The surrogate's BF16 training GEMMs on the tensor cores (mlp_gemm_tc.cu):
// C[z] = beta C[z] + opA[z] opB[z]^T with mlp.cu's strided operand view.
// Returns false, launching nothing, when the shape or strides are outside
// what it stages (then the SIMT kernel runs).  `part` (part_elems floats, may
// be null) is scratch for splitting K when there are few row tiles.
bool mlp_gemm_tc(cudaStream_t st, int Z, int M, int N, int K, const __nv_bfloat16 *A, int sAm,
                 int sAk, size_t zA, const __nv_bfloat16 *B, int sBn, int sBk, size_t zB,
                 const int *tile_sp, size_t sBsp, float *C, int ldc, size_t zC, float beta,
                 int *flags, float *part = nullptr, size_t part_elems = 0);
int kernel_occupancy(const void *fn, int threads, size_t smem);
int device_sms();

// variance.cu
gapgb_status variance_set_qmm(gapgb_model *m, const double *qmm);
bool variance_fp64_form(const gapgb_model *m);
size_t variance_tc_smem_bytes();
// covf of the N atoms (G: the descriptors of the last evaluation, FP64 when
// g64) and the per-structure VARIANCE into m->var.covf / m->var.var
gapgb_status variance_enqueue(gapgb_model *m, int S, int N, const int *d_atom_off, const void *G,
                              bool g64, cudaStream_t st);
void variance_free(VarState &v);

// model.cpp
gapgb_status parse_model_file(const char *path, HostModel *m, std::string *err);
gapgb_status write_model_file(const HostModel &m, const char *path, std::string *err);
gapgb_status build_sf_table(const HostModel &m, SFDev *t, std::string *err);

// api.cu
void set_last_error(const std::string &s);

// kernel launchers (nbr.cu, wacsf.cu, gpr.cu, reduce.cu)
void launch_prep(const gapgb_model *m, Workspace &ws, int S, int N, const int *d_atom_off,
                 const int *d_species, const double *d_lat, const double *d_pos,
                 double rcut, cudaStream_t st, bool allow_bins = false);
// exact: the reference's bit-identical list (FP64 path, neighbour export);
// otherwise the FP32 forms' cheaper geometry (same pairs up to last-bit
// decisions at r = rcut, where every term vanishes)
void launch_neighbors(Workspace &ws, int S, int N, int max_atoms, int cap, double rcut,
                      cudaStream_t st, bool exact = true);
void launch_reverse(Workspace &ws, int N, int cap, cudaStream_t st);
void launch_refresh(Workspace &ws, int N, int cap, cudaStream_t st, bool exact = true);
// [a0, a1) restricts the grouped FP32 kernels to a range of atoms (a1 < 0:
// up to N); the generic and FP64 kernels take the whole batch
template <typename T>
void launch_wacsf_fwd(const gapgb_model *m, Workspace &ws, int N, int cap, int cap_smem,
                      cudaStream_t st, int a0 = 0, int a1 = -1);
// whether the FP32 gradient kernel of this model scatters the forces itself
// (the reverse slots are then not needed)
bool bwd_scatters_forces(const gapgb_model *m);
// returns true when the kernel scattered the forces into d_force itself
// (grouped FP32 kernels); otherwise launch_forces gathers the slot gradients
// (zero_force: clear d_force first; a range call leaves that to its caller)
template <typename T>
bool launch_wacsf_bwd(const gapgb_model *m, Workspace &ws, int N, int cap, int cap_smem,
                      double *d_force, cudaStream_t st, int a0 = 0, int a1 = -1,
                      bool zero_force = true);
template <typename T, typename TG>
void launch_gpr(const gapgb_model *m, Workspace &ws, int N, cudaStream_t st);
// the tensor-core GPRs over atoms [a0, a1) of an N-atom batch (a0 a multiple
// of 128; a1 < 0: up to N)
void launch_gpr_tc(gapgb_model *m, Workspace &ws, int N, cudaStream_t st, int a0 = 0,
                   int a1 = -1);
template <typename T>
void launch_forces(Workspace &ws, int N, int cap, double *d_force, cudaStream_t st);
void launch_struct_reduce(Workspace &ws, int S, int lgrad, double *d_energy, double *d_stress,
                          double *d_atom_e, int N, cudaStream_t st);
void launch_min_bond(Workspace &ws, int N, double rcut, double *d_out, cudaStream_t st);
size_t wacsf_smem_bytes(const SFDev &t, int cap_smem, bool fwd, size_t elem);
int gpr_nsplit(int N, int M);
size_t gpr_scratch_bytes(int N, int M, int D, size_t elem);
// The tensor-core operand images: built by the first call that needs them;
// `refresh` rewrites an existing image in place (new coefficients) so that
// captured graphs keep valid addresses.
gapgb_status build_tc_image(gapgb_model *m, bool refresh = false);
size_t tc_atom_scratch_bytes(int N);
gapgb_status build_tf32_image(gapgb_model *m, bool refresh = false);
size_t tf32_atom_scratch_bytes(int N);
void launch_gpr_tf32(gapgb_model *m, Workspace &ws, int N, cudaStream_t st, int a0 = 0,
                     int a1 = -1);
void launch_gpr_rows(const gapgb_model *m, Workspace &ws, int cap, const int *d_rows,
                     const int *d_count, void *scratch, cudaStream_t st);
size_t gpr_rows_scratch_bytes(int cap, int D);

// api.cu, for md.cu
gapgb_status md_prepare(gapgb_model *m, int N, int S);
gapgb_status md_eval_enqueue(gapgb_model *m, int S, int N, const int *d_atom_off,
                             const int *d_species, const double *d_lat, const double *d_pos,
                             bool rebuild, double skin, double *d_energy, double *d_force,
                             double *d_stress, cudaStream_t s);
gapgb_status md_read_flags(gapgb_model *m, int *max_count);
gapgb_status md_clear_flags(gapgb_model *m);

// mlp.cu (learned surrogate)
gapgb_status surrogate_prepare(gapgb_surrogate *s, int N);
void surrogate_enqueue(gapgb_surrogate *s, int N, const int *d_Z, const float *d_G, double *d_e,
                       float *d_std, float *d_dedg, float *d_gstd, int *d_err, cudaStream_t st);
void surrogate_select_fallback(int N, const float *d_std, float threshold, const float *d_gstd,
                               float grad_spread, const int *d_cnt, const float4 *d_d32, int cap,
                               float r_contact, int *d_rows, int *d_count, cudaStream_t st);
int surrogate_device(const gapgb_surrogate *s);
// mlp_tc.cu (surrogate inference on the tensor cores)
bool mlp_tc_eligible(int D, int H);
size_t mlp_tc_w_image_bytes(int nblk);
size_t mlp_tc_x_image_bytes(int Mpad);
void launch_mlp_w_image(int nblk, int D, size_t P, size_t offW1, size_t offW2, size_t offb1,
                        size_t offb2, size_t offw3, size_t offb3, const __nv_bfloat16 *w16,
                        const float *w32, unsigned char *img, cudaStream_t st);
void launch_mlp_tc(int members, int nsp, int D, int Mpad, const unsigned char *wimg,
                   unsigned char *ximg, const int *idx, const float *G, const float *mu,
                   const float *isig, const int *tile_sp64, float *y, float *gx, int *flags,
                   cudaStream_t st);
int surrogate_des_len(const gapgb_surrogate *s);
bool surrogate_has_species(const gapgb_surrogate *s, int z);

}  // namespace gapgb

#define GAPGB_CUDA_TRY(expr)                                                      \
  do {                                                                            \
    cudaError_t _e = (expr);                                                      \
    if (_e != cudaSuccess) {                                                      \
      gapgb::set_last_error(std::string(#expr) + ": " + cudaGetErrorString(_e));  \
      return GAPGB_ERR_CUDA;                                                      \
    }                                                                             \
  } while (0)
