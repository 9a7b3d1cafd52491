// model.cpp - gap_parameters reader and symmetry-function table builder.
//
// File grammar (the reader of FGAP_READ, gappy/libgap/gap_calc.f90:303-364,
// the species read of FGAP_CALC, gap_calc.f90:75-83, and the SF read of
// CAR2ACSF, gappy/libgap/wacsf.f90:45-56), one Fortran record per line, read
// list-directed (blank/comma separated, r*v repeats, '/' ends a read, Fortran
// 'D' exponents):
//   nspecies
//   Z weight                 x nspecies
//   nsf
//   type alpha cutoff [zeta] x nsf    (zeta: optional extension, default 1)
//   M D
//   <3 records skipped>
//   theta(1:D)               (may span records)
//   MM(k,1:D)                x M, each starting a new record
//   coeff(1:M)
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "gapgb_internal.h"

namespace gapgb {
namespace {

class Records {
 public:
  explicit Records(std::vector<std::string> lines) : lines_(std::move(lines)) {}

  bool skip() {
    if (cur_ >= lines_.size()) return false;
    ++cur_;
    return true;
  }

  // Reads n values starting at the next record; returns the number of
  // unread tokens left on the last record consumed (or -1 on error).
  int read(int n, double *out) {
    int got = 0;
    int leftover = 0;
    while (got < n) {
      if (cur_ >= lines_.size()) return -1;
      const std::string &ln = lines_[cur_++];
      size_t p = 0;
      leftover = 0;
      while (p < ln.size()) {
        while (p < ln.size() && (std::isspace((unsigned char)ln[p]) || ln[p] == ',')) ++p;
        if (p >= ln.size()) break;
        if (ln[p] == '/') return got == n ? 0 : -1;
        size_t s = p;
        while (p < ln.size() && !std::isspace((unsigned char)ln[p]) && ln[p] != ',' && ln[p] != '/') ++p;
        std::string tok = ln.substr(s, p - s);
        if (got >= n) {
          ++leftover;
          continue;
        }
        int rep = 1;
        size_t star = tok.find('*');
        if (star != std::string::npos) {
          rep = std::atoi(tok.substr(0, star).c_str());
          tok = tok.substr(star + 1);
        }
        for (char &ch : tok)
          if (ch == 'd' || ch == 'D') ch = 'e';
        char *end = nullptr;
        double v = std::strtod(tok.c_str(), &end);
        if (tok.empty() || end != tok.c_str() + tok.size()) return -1;
        for (int q = 0; q < rep && got < n; ++q) out[got++] = v;
      }
    }
    return leftover;
  }

  size_t pos() const { return cur_; }
  void seek(size_t p) { cur_ = p; }

 private:
  std::vector<std::string> lines_;
  size_t cur_ = 0;
};

}  // namespace

gapgb_status parse_model_file(const char *path, HostModel *m, std::string *err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    *err = std::string("cannot open model file '") + path + "'";
    return GAPGB_ERR_FILE;
  }
  std::vector<std::string> lines;
  std::string ln;
  while (std::getline(f, ln)) {
    if (!ln.empty() && ln.back() == '\r') ln.pop_back();
    lines.push_back(ln);
  }
  Records r(std::move(lines));
  auto fail = [&](const char *what) {
    *err = std::string("gap_parameters: ") + what + " (record " + std::to_string(r.pos()) + ")";
    return GAPGB_ERR_PARSE;
  };
  double v[4];
  if (r.read(1, v) < 0) return fail("nspecies");
  m->nspecies = (int)v[0];
  if (m->nspecies <= 0 || m->nspecies > 118) return fail("nspecies out of range");
  m->species_z.assign(m->nspecies, 0);
  m->species_w.assign(m->nspecies, 0.0);
  for (int i = 0; i < m->nspecies; ++i) {
    if (r.read(2, v) < 0) return fail("species record");
    m->species_z[i] = (int)v[0];
    m->species_w[i] = v[1];
  }
  if (r.read(1, v) < 0) return fail("nsf");
  m->nsf = (int)v[0];
  if (m->nsf <= 0 || m->nsf > kMaxSF) return fail("nsf out of range");
  m->sf_type.assign(m->nsf, 0);
  m->sf_alpha.assign(m->nsf, 0.0);
  m->sf_cutoff.assign(m->nsf, 0.0);
  m->sf_zeta.assign(m->nsf, 1.0);
  for (int i = 0; i < m->nsf; ++i) {
    size_t p0 = r.pos();
    int left = r.read(3, v);
    if (left < 0) return fail("SF record");
    m->sf_type[i] = (int)v[0];
    m->sf_alpha[i] = v[1];
    m->sf_cutoff[i] = v[2];
    if (left > 0 && r.pos() == p0 + 1) {
      r.seek(p0);
      if (r.read(4, v) < 0) return fail("SF zeta column");
      m->sf_zeta[i] = v[3];
    }
  }
  if (r.read(2, v) < 0) return fail("M D record");
  m->M = (int)v[0];
  m->D = (int)v[1];
  if (m->M <= 0 || m->D <= 0) return fail("M or D not positive");
  for (int i = 0; i < 3; ++i)
    if (!r.skip()) return fail("missing records after M D");
  m->theta.assign(m->D, 0.0);
  m->mm.assign((size_t)m->M * m->D, 0.0);
  m->coeff.assign(m->M, 0.0);
  if (r.read(m->D, m->theta.data()) < 0) return fail("theta");
  for (int k = 0; k < m->M; ++k)
    if (r.read(m->D, m->mm.data() + (size_t)k * m->D) < 0) return fail("sparse point row");
  if (r.read(m->M, m->coeff.data()) < 0) return fail("coeff");
  return GAPGB_OK;
}

// Writes a model in the grammar above, every value as %.17g so that a read
// gives back the same doubles.  The zeta column appears only on SF records
// whose zeta differs from 1, so a file of the reference's own SF types is
// one FGAP_READ / CAR2ACSF can read unchanged; the three records after
// "M D" are left blank (FGAP_READ skips them, gap_calc.f90:352-354).
gapgb_status write_model_file(const HostModel &m, const char *path, std::string *err) {
  std::FILE *f = std::fopen(path, "w");
  if (!f) {
    *err = std::string("cannot create model file '") + path + "'";
    return GAPGB_ERR_FILE;
  }
  std::fprintf(f, "%d\n", m.nspecies);
  for (int i = 0; i < m.nspecies; ++i) std::fprintf(f, "%6d %.17g\n", m.species_z[i], m.species_w[i]);
  std::fprintf(f, "%d\n", m.nsf);
  for (int i = 0; i < m.nsf; ++i) {
    if (m.sf_zeta[i] != 1.0)
      std::fprintf(f, "%d %.17g %.17g %.17g\n", m.sf_type[i], m.sf_alpha[i], m.sf_cutoff[i],
                   m.sf_zeta[i]);
    else
      std::fprintf(f, "%d %.17g %.17g\n", m.sf_type[i], m.sf_alpha[i], m.sf_cutoff[i]);
  }
  std::fprintf(f, "%d %d\n\n\n\n", m.M, m.D);
  auto row = [&](const double *v, int n) {
    for (int q = 0; q < n; ++q) std::fprintf(f, q ? " %.17g" : "%.17g", v[q]);
    std::fputc('\n', f);
  };
  row(m.theta.data(), m.D);
  for (int k = 0; k < m.M; ++k) row(m.mm.data() + (size_t)k * m.D, m.D);
  row(m.coeff.data(), m.M);
  const bool bad = std::ferror(f) != 0;
  if (std::fclose(f) != 0 || bad) {
    *err = std::string("write error on model file '") + path + "'";
    return GAPGB_ERR_FILE;
  }
  return GAPGB_OK;
}

gapgb_status build_sf_table(const HostModel &m, SFDev *t, std::string *err) {
  std::memset(t, 0, sizeof(*t));
  t->nsf = m.nsf;
  t->D = m.D;
  if (2 * m.nsf > m.D) {
    *err = "descriptor length D must be at least 2*nsf (wacsf.f90:86-87 writes d and d+nsf)";
    return GAPGB_ERR_PARSE;
  }
  auto rc_index = [&](double rc) -> int {
    for (int q = 0; q < t->nrc; ++q)
      if (t->rc_val[q] == rc) return q;
    if (t->nrc >= kMaxRC) return -1;
    t->rc_val[t->nrc] = rc;
    return t->nrc++;
  };
  auto alpha_index = [&](double a) -> int {
    for (int q = 0; q < t->nalpha; ++q)
      if (t->alpha_val[q] == a) return q;
    if (t->nalpha >= kMaxAlpha) return -1;
    t->alpha_val[t->nalpha] = a;
    return t->nalpha++;
  };
  struct Ang { int d, rc, al; double lam, zeta; };
  std::vector<Ang> ang;
  for (int s = 0; s < m.nsf; ++s) {
    const int ty = m.sf_type[s];
    const double rc = m.sf_cutoff[s];
    if (!(rc > 0.0)) {
      *err = "SF cutoff must be positive";
      return GAPGB_ERR_PARSE;
    }
    if (ty == 1 || ty == 3) {
      int q = t->nrad++;
      t->rad_d[q] = s;
      t->rad_rc[q] = rc_index(rc);
      t->rad_alpha[q] = (ty == 1) ? m.sf_alpha[s] : 4.0;
      t->rad_rs[q] = (ty == 1) ? 0.0 : m.sf_alpha[s];
      if (t->rad_rc[q] < 0) { *err = "too many distinct SF cutoffs"; return GAPGB_ERR_CAP_EXCEEDED; }
      if (rc > t->max_rc) t->max_rc = rc;
    } else if (ty == 2 || ty == 4) {
      Ang a;
      a.d = s;
      a.rc = rc_index(rc);
      a.al = alpha_index(m.sf_alpha[s]);
      a.lam = (ty == 2) ? 1.0 : -1.0;
      a.zeta = m.sf_zeta[s];
      if (a.rc < 0 || a.al < 0) { *err = "too many distinct angular cutoffs or alphas"; return GAPGB_ERR_CAP_EXCEEDED; }
      if (!(a.zeta > 0.0)) { *err = "angular zeta must be positive"; return GAPGB_ERR_PARSE; }
      ang.push_back(a);
      if (rc > t->max_ang_rc) t->max_ang_rc = rc;
      if (rc > t->max_rc) t->max_rc = rc;
    }
    // other types: the reference leaves the entries at zero (wacsf.f90:792-794)
  }
  // group angular SFs by cutoff index (stable: descriptor order within a group)
  t->nang = (int)ang.size();
  int q = 0;
  t->n_ang_grp = 0;
  for (int rc = 0; rc < t->nrc; ++rc) {
    int start = q;
    for (const Ang &a : ang) {
      if (a.rc != rc) continue;
      t->ang_d[q] = a.d;
      t->ang_rc[q] = a.rc;
      t->ang_alpha[q] = a.al;
      t->ang_lambda[q] = a.lam;
      t->ang_zeta[q] = a.zeta;
      double zr = std::nearbyint(a.zeta);
      t->ang_izeta[q] = (zr == a.zeta && zr >= 1 && zr <= 16) ? (int)zr : -1;
      t->ang_pref[q] = std::pow(2.0, 1.0 - a.zeta);
      ++q;
    }
    if (q > start) {
      t->ang_grp_rc[t->n_ang_grp] = rc;
      t->ang_grp_start[t->n_ang_grp] = start;
      ++t->n_ang_grp;
    }
  }
  t->ang_grp_start[t->n_ang_grp] = q;
  if (m.nspecies > kMaxSpecies) {
    *err = "too many species";
    return GAPGB_ERR_CAP_EXCEEDED;
  }
  t->nspecies = m.nspecies;
  for (int i = 0; i < m.nspecies; ++i) {
    t->species_z[i] = m.species_z[i];
    t->species_w[i] = m.species_w[i];
  }
  return GAPGB_OK;
}

}  // namespace gapgb
