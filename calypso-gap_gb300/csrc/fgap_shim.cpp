// fgap_shim.cpp - the reference's Fortran entry points with the gfortran ABI.
//
// calypso-side callers (calypso.x, GULP "nnpcal", ngap.x) call
//   FGAP_READ(nsparseX, des_len, theta(100), MM(4000,100), invcmm(4000,4000), coeff(4000))
//   FGAP_CALC(NA, SPECIES, LAT, POS, ENE, FORCE, STRESS, VARIANCE,
//             nsparseX, des_len, theta, MM, qmm, coeff, Rcut, lgrad)
//   FGET_BOND(na, lat, elements, pos, rcut, min_bond)
// (gappy/libgap/gap_calc.f90:1-46, :303-314; gappy/libgap/get_bond.f90:4-13).
// gfortran passes every argument by reference, LOGICAL as a 4-byte integer,
// and arrays column-major: POS(i,k) is pos[i + NA*k], LAT(i,j) is
// lat[i + 3*j] with LAT(i,:) = lattice vector i, MM(k,d) is mm[k + M*d].
// These symbols (fgap_read_, fgap_calc_, fget_bond_) link in place of the
// Fortran objects; like the reference they read ./gap_parameters for the
// species weights and the SF table.  They never stop the process: failures
// are printed to stderr and leave the outputs zeroed (FGAP_READ sets
// nsparseX = 0).
#include <sys/stat.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "gapgb_internal.h"

namespace {

constexpr int kNsfMax = 100;       // gap_calc.f90:306
constexpr int kSparseMax = 4000;   // gap_calc.f90:307

struct ShimCache {
  gapgb_model *model = nullptr;
  long long mtime = -1, size = -1;
  int M = 0, D = 0;
  double rcut = 0;
  std::vector<double> theta, mm, coeff;  // as last uploaded (row-major mm)
};

std::mutex g_mu;
ShimCache g_cache;

bool file_stamp(long long *mtime, long long *size) {
  struct stat st;
  if (stat("gap_parameters", &st) != 0) return false;
  *mtime = (long long)st.st_mtime;
  *size = (long long)st.st_size;
  return true;
}

void report(const char *where) {
  std::fprintf(stderr, "%s: %s\n", where, gapgb_last_error());
}

}  // namespace

extern "C" {

void fgap_read_(int *nsparseX, int *des_len, double *theta, double *MM, double *invcmm,
                double *coeff) {
  std::lock_guard<std::mutex> lock(g_mu);
  *nsparseX = 0;
  *des_len = 0;
  gapgb::HostModel h;
  std::string err;
  if (gapgb::parse_model_file("gap_parameters", &h, &err) != GAPGB_OK) {
    std::fprintf(stderr, "fgap_read: %s\n", err.c_str());
    return;
  }
  if (h.M > kSparseMax || h.D > kNsfMax) {
    std::fprintf(stderr, "fgap_read: M=%d D=%d exceed the fixed arrays (4000, 100); use gapgb_model_load\n",
                 h.M, h.D);
    return;
  }
  std::memset(theta, 0, sizeof(double) * kNsfMax);
  std::memset(MM, 0, sizeof(double) * kSparseMax * kNsfMax);
  std::memset(invcmm, 0, sizeof(double) * (size_t)kSparseMax * kSparseMax);  // gap_calc.f90:361
  std::memset(coeff, 0, sizeof(double) * kSparseMax);
  for (int d = 0; d < h.D; ++d) theta[d] = h.theta[d];
  for (int k = 0; k < h.M; ++k)
    for (int d = 0; d < h.D; ++d) MM[k + (size_t)kSparseMax * d] = h.mm[(size_t)k * h.D + d];
  for (int k = 0; k < h.M; ++k) coeff[k] = h.coeff[k];
  *nsparseX = h.M;
  *des_len = h.D;
}

void fgap_calc_(const int *NA, const int *SPECIES, const double *LAT, const double *POS,
                double *ENE, double *FORCE, double *STRESS, double *VARIANCE,
                const int *nsparseX, const int *des_len, const double *theta, const double *MM,
                const double *qmm, const double *coeff, const double *Rcut, const int *lgrad) {
  (void)qmm;  // the reference never reads it (variance is 0, gap_calc.f90:206-210)
  std::lock_guard<std::mutex> lock(g_mu);
  const int na = *NA, M = *nsparseX, D = *des_len;
  *ENE = 0.0;
  *VARIANCE = 0.0;
  std::memset(FORCE, 0, sizeof(double) * 3 * (size_t)(na > 0 ? na : 0));
  std::memset(STRESS, 0, sizeof(double) * 6);
  if (na <= 0 || M <= 0 || D <= 0) {
    std::fprintf(stderr, "fgap_calc: invalid sizes\n");
    return;
  }
  // model arrays in row-major form
  std::vector<double> th(theta, theta + D), mm((size_t)M * D), co(coeff, coeff + M);
  for (int k = 0; k < M; ++k)
    for (int d = 0; d < D; ++d) mm[(size_t)k * D + d] = MM[k + (size_t)M * d];
  long long mt = -1, sz = -1;
  if (!file_stamp(&mt, &sz)) {
    std::fprintf(stderr, "fgap_calc: gap_parameters file does not exist!\n");
    return;
  }
  ShimCache &c = g_cache;
  const bool same = c.model && c.mtime == mt && c.size == sz && c.M == M && c.D == D &&
                    c.rcut == *Rcut && c.theta == th && c.mm == mm && c.coeff == co;
  if (!same) {
    if (c.model) gapgb_model_free(c.model);
    c.model = nullptr;
    gapgb::HostModel h;
    std::string err;
    if (gapgb::parse_model_file("gap_parameters", &h, &err) != GAPGB_OK) {
      std::fprintf(stderr, "fgap_calc: %s\n", err.c_str());
      return;
    }
    gapgb_model *m = nullptr;
    if (gapgb_model_create(h.nspecies, h.species_z.data(), h.species_w.data(), h.nsf,
                           h.sf_type.data(), h.sf_alpha.data(), h.sf_cutoff.data(),
                           h.sf_zeta.data(), M, D, th.data(), mm.data(), co.data(), *Rcut,
                           &m) != GAPGB_OK) {
      report("fgap_calc");
      return;
    }
    c.model = m;
    c.mtime = mt;
    c.size = sz;
    c.M = M;
    c.D = D;
    c.rcut = *Rcut;
    c.theta = th;
    c.mm = mm;
    c.coeff = co;
  }
  double lat[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) lat[i * 3 + j] = LAT[i + 3 * j];
  std::vector<double> pos((size_t)na * 3), force((size_t)na * 3);
  for (int i = 0; i < na; ++i)
    for (int k = 0; k < 3; ++k) pos[(size_t)i * 3 + k] = POS[i + (size_t)na * k];
  double stress[6], var = 0.0;
  if (gapgb_eval(c.model, na, SPECIES, lat, pos.data(), *lgrad ? 1 : 0, ENE, force.data(), stress,
                 &var) != GAPGB_OK) {
    report("fgap_calc");
    *ENE = 0.0;
    return;
  }
  for (int i = 0; i < na; ++i)
    for (int k = 0; k < 3; ++k) FORCE[i + (size_t)na * k] = force[(size_t)i * 3 + k];
  for (int q = 0; q < 6; ++q) STRESS[q] = stress[q];
  *VARIANCE = var;
}

void fget_bond_(const int *na, const double *lat_f, const int *elements, const double *pos_f,
                const double *rcut, double *min_bond) {
  (void)elements;
  const int n = *na;
  *min_bond = 10.0;
  if (n <= 0) return;
  double lat[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) lat[i * 3 + j] = lat_f[i + 3 * j];
  std::vector<double> pos((size_t)n * 3);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) pos[(size_t)i * 3 + k] = pos_f[i + (size_t)n * k];
  if (gapgb_min_bond(n, lat, pos.data(), *rcut, min_bond) != GAPGB_OK) report("fget_bond");
}

}  // extern "C"
