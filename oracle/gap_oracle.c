/*
 * gap_oracle.c - CPU FP64 restatement of CALYPSO-GAP's FGAP_CALC / CAR2ACSF /
 * FGAP_READ / FGET_BOND.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle for the CUDA product path and the
 * CPU baseline timed by bench.py.  Nothing in the product links or calls it.
 *
 * Pinned against the reference's own outputs: the 11 frames of
 * gappy/example/ASE-GAPPY/ase.traj (energy, forces and stress written by the
 * reference through ASE) with the model gappy/example/ASE-GAPPY/gap_parameters.
 *
 * Every loop follows the Fortran statement by statement, including the
 * truncated pi = 3.141592654 (gap_calc.f90:59, wacsf.f90:31), the '>' cutoff
 * tests, the j -> n1 -> n2 -> n3 neighbour order, the dense Jacobian dxdy and
 * the upper-triangle stress.  Build with -ffp-contract=off so that every
 * Fortran expression is evaluated with separately rounded operations in
 * left-to-right order.
 *
 * Extension (absent from the reference, which reads and ignores a 4th column
 * on SF lines): angular types 2 and 4 take an optional zeta column and then
 * use 2^(1-zeta) (1 +- cos)^zeta.  zeta == 1 is the reference formula.
 */
#include "gap_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double ORC_PI = 3.141592654; /* gap_calc.f90:59, wacsf.f90:31 */
static const double ORC_DELTA = 1.0;      /* gap_calc.f90:8 */
static const double ORC_GPA2EVPANG = 6.24219e-3; /* gap_calc.f90:9 */

/* ------------------------------------------------------------------------ */
/* Fortran list-directed input over a file held as lines.                   */
/* ------------------------------------------------------------------------ */
typedef struct {
  char **line;
  int nline;
  int cur;
} rec_reader;

static int rr_open(const char *path, rec_reader *r) {
  FILE *f = fopen(path, "rb");
  if (!f) return ORC_ERR_FILE;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  char *buf = (char *)malloc((size_t)n + 1);
  if (!buf) { fclose(f); return ORC_ERR_ALLOC; }
  if (n > 0 && fread(buf, 1, (size_t)n, f) != (size_t)n) { fclose(f); free(buf); return ORC_ERR_FILE; }
  fclose(f);
  buf[n] = 0;
  int cap = 1024;
  r->line = (char **)malloc(sizeof(char *) * cap);
  r->nline = 0;
  r->cur = 0;
  char *p = buf;
  while (*p) {
    char *e = strchr(p, '\n');
    if (r->nline == cap) { cap *= 2; r->line = (char **)realloc(r->line, sizeof(char *) * cap); }
    r->line[r->nline++] = p;
    if (!e) break;
    *e = 0;
    p = e + 1;
  }
  if (r->nline == 0) { r->line[0] = buf; r->nline = 0; }
  /* keep buf alive through line[0]; freed in rr_close */
  r->line = (char **)realloc(r->line, sizeof(char *) * (r->nline + 1));
  r->line[r->nline] = buf;
  return ORC_OK;
}

static void rr_close(rec_reader *r) {
  if (r->line) { free(r->line[r->nline]); free(r->line); }
  r->line = NULL;
}

/* read(u,*) with an empty list: skip one record */
static int rr_skip(rec_reader *r) {
  if (r->cur >= r->nline) return ORC_ERR_PARSE;
  r->cur++;
  return ORC_OK;
}

/* Parse one value token (handles Fortran D exponents). */
static int parse_value(const char *tok, int len, double *v) {
  char tmp[96];
  if (len <= 0 || len >= (int)sizeof(tmp)) return 0;
  for (int i = 0; i < len; i++) tmp[i] = (tok[i] == 'd' || tok[i] == 'D') ? 'e' : tok[i];
  tmp[len] = 0;
  char *end;
  *v = strtod(tmp, &end);
  return end == tmp + len;
}

/* read(u,*) v(1:n): n values from successive records, rest of last record
 * discarded.  Separators: blanks and commas; 'r*v' repeat counts; '/' ends. */
static int rr_read(rec_reader *r, int n, double *out, int *ntok_last) {
  int got = 0;
  while (got < n) {
    if (r->cur >= r->nline) return ORC_ERR_PARSE;
    const char *p = r->line[r->cur++];
    int on_line = 0;
    while (*p && got < n) {
      while (*p && (isspace((unsigned char)*p) || *p == ',')) p++;
      if (!*p) break;
      if (*p == '/') return got == n ? ORC_OK : ORC_ERR_PARSE;
      const char *s = p;
      while (*p && !isspace((unsigned char)*p) && *p != ',' && *p != '/') p++;
      int len = (int)(p - s);
      const char *star = memchr(s, '*', (size_t)len);
      int rep = 1;
      if (star) {
        rep = atoi(s);
        len -= (int)(star + 1 - s);
        s = star + 1;
      }
      double v;
      if (!parse_value(s, len, &v)) return ORC_ERR_PARSE;
      for (int q = 0; q < rep && got < n; q++) out[got++] = v;
      on_line++;
    }
    if (ntok_last) {
      /* count the remaining tokens of this record (used for the optional
       * zeta column on SF lines) */
      int extra = 0;
      while (*p) {
        while (*p && (isspace((unsigned char)*p) || *p == ',')) p++;
        if (!*p) break;
        extra++;
        while (*p && !isspace((unsigned char)*p) && *p != ',') p++;
      }
      *ntok_last = extra;
    }
  }
  return ORC_OK;
}

/* FGAP_READ (gap_calc.f90:303-364) plus the species table
 * (gap_calc.f90:75-83) and the SF table (wacsf.f90:45-56).  The reference's
 * fixed caps (M <= 4000, D <= 100, gap_calc.f90:341-350) are not applied
 * here; the product's reference-compatible fgap_read applies them. */
int orc_model_read(const char *path, orc_model *m) {
  memset(m, 0, sizeof(*m));
  rec_reader r;
  int st = rr_open(path, &r);
  if (st) return st;
  double v[8];
  st = ORC_ERR_PARSE;
  if (rr_read(&r, 1, v, NULL)) goto done;
  m->nspecies = (int)v[0];
  if (m->nspecies < 0 || m->nspecies > 128) goto done;
  for (int i = 0; i < m->nspecies; i++) {
    if (rr_read(&r, 2, v, NULL)) goto done;
    m->species_z[i] = (int)v[0];
    m->species_w[i] = v[1];
  }
  if (rr_read(&r, 1, v, NULL)) goto done;
  m->nsf = (int)v[0];
  if (m->nsf < 0 || m->nsf > 256) goto done;
  for (int i = 0; i < m->nsf; i++) {
    /* read the whole record so that an optional 4th column can be seen */
    if (r.cur >= r.nline) goto done;
    int save = r.cur;
    int extra = 0;
    if (rr_read(&r, 3, v, &extra)) goto done;
    m->sf_type[i] = (int)v[0];
    m->sf_alpha[i] = v[1];
    m->sf_cutoff[i] = v[2];
    m->sf_zeta[i] = 1.0;
    if (extra > 0 && r.cur == save + 1) {
      r.cur = save;
      double w4[4];
      if (rr_read(&r, 4, w4, NULL)) goto done;
      m->sf_zeta[i] = w4[3];
    }
  }
  if (rr_read(&r, 2, v, NULL)) goto done;
  m->nsparse = (int)v[0];
  m->des_len = (int)v[1];
  if (m->nsparse <= 0 || m->des_len <= 0) goto done;
  for (int i = 0; i < 3; i++)
    if (rr_skip(&r)) goto done;
  m->theta = (double *)malloc(sizeof(double) * m->des_len);
  m->mm = (double *)malloc(sizeof(double) * (size_t)m->nsparse * m->des_len);
  m->coeff = (double *)malloc(sizeof(double) * m->nsparse);
  if (!m->theta || !m->mm || !m->coeff) { st = ORC_ERR_ALLOC; goto done; }
  if (rr_read(&r, m->des_len, m->theta, NULL)) goto done;
  for (int k = 0; k < m->nsparse; k++)
    if (rr_read(&r, m->des_len, m->mm + (size_t)k * m->des_len, NULL)) goto done;
  if (rr_read(&r, m->nsparse, m->coeff, NULL)) goto done;
  st = ORC_OK;
done:
  rr_close(&r);
  if (st) orc_model_free(m);
  return st;
}

void orc_model_free(orc_model *m) {
  free(m->theta);
  free(m->mm);
  free(m->coeff);
  m->theta = m->mm = m->coeff = NULL;
}

/* ------------------------------------------------------------------------ */
/* Lattice helpers, gap_calc.f90:235-266 and 290-299.  Fortran LAT(i,j) is  */
/* lat[(i-1)*3+(j-1)] here.                                                 */
/* ------------------------------------------------------------------------ */
#define LAT(i, j) lat[((i) - 1) * 3 + ((j) - 1)]

static void crossp(const double *va, const double *vb, double *out) {
  out[0] = va[1] * vb[2] - va[2] * vb[1];
  out[1] = va[2] * vb[0] - va[0] * vb[2];
  out[2] = va[0] * vb[1] - va[1] * vb[0];
}

static double lat_volume(const double *lat) {
  double c1[3] = {LAT(1, 1), LAT(2, 1), LAT(3, 1)};
  double c2[3] = {LAT(1, 2), LAT(2, 2), LAT(3, 2)};
  double c3[3] = {LAT(1, 3), LAT(2, 3), LAT(3, 3)};
  double x[3];
  crossp(c2, c3, x);
  return fabs(c1[0] * x[0] + c1[1] * x[1] + c1[2] * x[2]);
}

void orc_nabc(const double *lat, double rcut, int nabc[3]) {
  double c1[3] = {LAT(1, 1), LAT(2, 1), LAT(3, 1)};
  double c2[3] = {LAT(1, 2), LAT(2, 2), LAT(3, 2)};
  double c3[3] = {LAT(1, 3), LAT(2, 3), LAT(3, 3)};
  double rc[3][3]; /* rc[col][row] = recipvector(row, col) */
  crossp(c2, c3, rc[0]);
  crossp(c3, c1, rc[1]);
  crossp(c1, c2, rc[2]);
  double vol = lat_volume(lat);
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) rc[a][b] = rc[a][b] / vol * ORC_PI * 2.0;
  for (int row = 0; row < 3; row++) {
    double x = rc[0][row], y = rc[1][row], z = rc[2][row];
    double len = sqrt(x * x + y * y + z * z);
    nabc[row] = (int)ceil(rcut * len / ORC_PI / 2);
  }
}

static double lat_det(const double *lat) {
  return LAT(1, 1) * (LAT(2, 2) * LAT(3, 3) - LAT(2, 3) * LAT(3, 2))
       - LAT(1, 2) * (LAT(2, 1) * LAT(3, 3) - LAT(2, 3) * LAT(3, 1))
       + LAT(1, 3) * (LAT(2, 1) * LAT(3, 2) - LAT(3, 1) * LAT(2, 2));
}

/* gap_calc.f90:85-120 */
int orc_neighbors(int na, const double *lat, const double *pos,
                  const double *weights, double rcut, int max_nb,
                  int *count, double *nb) {
  int nabc[3];
  orc_nabc(lat, rcut, nabc);
  for (int i = 0; i < na; i++) count[i] = 0;
  for (int i = 0; i < na; i++) {
    for (int j = 0; j < na; j++) {
      for (int n1 = -nabc[0]; n1 <= nabc[0]; n1++)
        for (int n2 = -nabc[1]; n2 <= nabc[1]; n2++)
          for (int n3 = -nabc[2]; n3 <= nabc[2]; n3++) {
            if (n1 == 0 && n2 == 0 && n3 == 0 && i == j) continue;
            double xyz[3], dr[3];
            for (int c = 0; c < 3; c++)
              xyz[c] = pos[j * 3 + c] + (double)n1 * lat[0 * 3 + c]
                     + (double)n2 * lat[1 * 3 + c] + (double)n3 * lat[2 * 3 + c];
            for (int c = 0; c < 3; c++) dr[c] = pos[i * 3 + c] - xyz[c];
            double dis = sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
            if (dis > rcut) continue;
            int k = count[i]++;
            if (count[i] > max_nb) return ORC_ERR_NEIGHBOUR_OVERFLOW;
            double *e = nb + ((size_t)i * max_nb + k) * 6;
            e[0] = xyz[0];
            e[1] = xyz[1];
            e[2] = xyz[2];
            e[3] = dis;
            e[4] = weights[j];
            e[5] = (double)(j + 1);
          }
    }
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* CAR2ACSF, wacsf.f90:2-796                                                 */
/* ------------------------------------------------------------------------ */
int orc_car2acsf(const orc_model *m, int na, int max_nb, const double *pos,
                 const double *nb, const int *count, double *xx,
                 double *dxdy, double *strs, int lgrad) {
  const int D = m->des_len, nnn = m->nsf;
  if (2 * nnn > D) return ORC_ERR_ARG;
  const double pi = ORC_PI;
  if (!dxdy || !strs) lgrad = 0;
#define XX(d, i) xx[(size_t)(i) * D + (d)]
#define DXDY(d, i, j, c) dxdy[(((size_t)(c) * na + (j)) * na + (i)) * D + (d)]
#define STRS(a, b, d, i) strs[(((size_t)(i) * D + (d)) * 3 + (b)) * 3 + (a)]
#define NB(i, k, f) nb[((size_t)(i) * max_nb + (k)) * 6 + (f)]
  memset(xx, 0, sizeof(double) * (size_t)na * D);
  if (lgrad) {
    memset(dxdy, 0, sizeof(double) * (size_t)D * na * na * 3);
    memset(strs, 0, sizeof(double) * (size_t)9 * D * na);
  }
  for (int ii = 0; ii < nnn; ii++) {
    const int type = m->sf_type[ii];
    const double cutoff = m->sf_cutoff[ii];
    if (type == 1 || type == 3) {
      /* G1 = sum_j exp(-alpha rij^2) fc(rij)          wacsf.f90:69-162
       * G3 = sum_j exp(-4 (rij - rs)^2) fc(rij)       wacsf.f90:436-527 */
      const double alpha = (type == 1) ? m->sf_alpha[ii] : 4.0;
      const double rshift = m->sf_alpha[ii];
      for (int i = 0; i < na; i++) {
        for (int q = 0; q < count[i]; q++) {
          double rij = NB(i, q, 3);
          if (rij > cutoff) continue;
          double xyz[3] = {NB(i, q, 0), NB(i, q, 1), NB(i, q, 2)};
          double weights = NB(i, q, 4);
          int n = (int)NB(i, q, 5) - 1;
          double fcutij = 0.5 * (cos(pi * rij / cutoff) + 1.0);
          double ex, t1;
          if (type == 1) {
            ex = exp(-1.0 * alpha * (rij * rij));
          } else {
            double u = rij - rshift;
            ex = exp(-1.0 * alpha * (u * u));
          }
          XX(ii, i) = XX(ii, i) + ex * fcutij;
          XX(ii + nnn, i) = XX(ii + nnn, i) + ex * fcutij * weights;
          if (!lgrad) continue;
          double delta[3], drdi[3], drdj[3], dfdi[3], dfdj[3];
          for (int c = 0; c < 3; c++) delta[c] = -1.0 * (pos[i * 3 + c] - xyz[c]);
          for (int c = 0; c < 3; c++) drdi[c] = -1.0 * delta[c] / rij;
          for (int c = 0; c < 3; c++) drdj[c] = -1.0 * drdi[c];
          double tc = 0.5 * (-sin(pi * rij / cutoff)) * (pi / cutoff);
          for (int c = 0; c < 3; c++) dfdi[c] = tc * drdi[c];
          for (int c = 0; c < 3; c++) dfdj[c] = -1.0 * dfdi[c];
          for (int c = 0; c < 3; c++) {
            double vi, t3;
            if (type == 1) {
              t1 = -2.0 * alpha * rij * ex * fcutij;
              vi = drdi[c] * t1 + ex * dfdi[c];
              t3 = drdj[c] * t1 + ex * dfdj[c];
            } else {
              t1 = -2.0 * alpha * (rij - rshift);
              vi = t1 * drdi[c] * ex * fcutij + ex * dfdi[c];
              t3 = t1 * drdj[c] * ex * fcutij + ex * dfdj[c];
            }
            DXDY(ii, i, i, c) = DXDY(ii, i, i, c) + vi;
            DXDY(ii + nnn, i, i, c) = DXDY(ii + nnn, i, i, c) + vi * weights;
            DXDY(ii, i, n, c) = DXDY(ii, i, n, c) + t3;
            double t4 = t3 * weights;
            DXDY(ii + nnn, i, n, c) = DXDY(ii + nnn, i, n, c) + t4;
            for (int a = 0; a < 3; a++) {
              STRS(a, c, ii, i) = STRS(a, c, ii, i) + delta[a] * t3;
              STRS(a, c, ii + nnn, i) = STRS(a, c, ii + nnn, i) + delta[a] * t4;
            }
          }
        }
      }
    } else if (type == 2 || type == 4) {
      /* G2/G4 = sum_{j<k} (1 +- cos theta_ijk) exp(-alpha (rij^2+rik^2+rjk^2))
       *         fc(rij) fc(rik) fc(rjk)            wacsf.f90:169-432, 534-791 */
      const double alpha = m->sf_alpha[ii];
      const double zeta = m->sf_zeta[ii];
      const double lam = (type == 2) ? 1.0 : -1.0;
      for (int i = 0; i < na; i++) {
        for (int jq = 0; jq < count[i]; jq++) {
          double rij = NB(i, jq, 3);
          if (rij > cutoff) continue;
          double xyzj[3] = {NB(i, jq, 0), NB(i, jq, 1), NB(i, jq, 2)};
          double fcutij = 0.5 * (cos(pi * rij / cutoff) + 1.0);
          double wj = NB(i, jq, 4);
          int n = (int)NB(i, jq, 5) - 1;
          /* role index r: 0 = atom i, 1 = atom j, 2 = atom k */
          double dj[3], drij[3][3], dfij[3][3];
          if (lgrad) {
            for (int c = 0; c < 3; c++) dj[c] = -1.0 * (pos[i * 3 + c] - xyzj[c]);
            for (int c = 0; c < 3; c++) {
              drij[0][c] = -1.0 * dj[c] / rij;
              drij[1][c] = -1.0 * drij[0][c];
              drij[2][c] = 0.0;
            }
            double tc = 0.5 * (-sin(pi * rij / cutoff)) * (pi / cutoff);
            for (int c = 0; c < 3; c++) {
              dfij[0][c] = tc * drij[0][c];
              dfij[1][c] = -1.0 * dfij[0][c];
              dfij[2][c] = 0.0;
            }
          }
          for (int kq = jq + 1; kq < count[i]; kq++) {
            double rik = NB(i, kq, 3);
            if (rik > cutoff) continue;
            double xyzk[3] = {NB(i, kq, 0), NB(i, kq, 1), NB(i, kq, 2)};
            double wk = NB(i, kq, 4);
            int mm = (int)NB(i, kq, 5) - 1;
            double fcutik = 0.5 * (cos(pi * rik / cutoff) + 1.0);
            double dk[3], drik[3][3], dfik[3][3];
            if (lgrad) {
              for (int c = 0; c < 3; c++) dk[c] = -1.0 * (pos[i * 3 + c] - xyzk[c]);
              for (int c = 0; c < 3; c++) {
                drik[0][c] = -dk[c] / rik;
                drik[2][c] = -1.0 * drik[0][c];
                drik[1][c] = 0.0;
              }
              double tc = 0.5 * (-sin(pi * rik / cutoff)) * (pi / cutoff);
              for (int c = 0; c < 3; c++) {
                dfik[0][c] = tc * drik[0][c];
                dfik[1][c] = 0.0;
                dfik[2][c] = -1.0 * dfik[0][c];
              }
            }
            double ax = xyzj[0] - xyzk[0], ay = xyzj[1] - xyzk[1], az = xyzj[2] - xyzk[2];
            double rjk = ax * ax + ay * ay + az * az;
            rjk = sqrt(rjk);
            if (rjk > cutoff) continue;
            double fcutjk = 0.5 * (cos(pi * rjk / cutoff) + 1.0);
            double drjk[3][3], dfjk[3][3];
            if (lgrad) {
              double dd[3] = {ax, ay, az};
              for (int c = 0; c < 3; c++) {
                drjk[1][c] = dd[c] / rjk;
                drjk[2][c] = -1.0 * drjk[1][c];
                drjk[0][c] = 0.0;
              }
              double tc = 0.5 * (-sin(pi * rjk / cutoff)) * (pi / cutoff);
              for (int c = 0; c < 3; c++) {
                dfjk[1][c] = tc * drjk[1][c];
                dfjk[2][c] = -1.0 * dfjk[1][c];
                dfjk[0][c] = 0.0;
              }
            }
            double f = rjk * rjk - rij * rij - rik * rik;
            double g = -2.0 * rij * rik;
            double costheta = f / g;
            costheta = (type == 2) ? 1.0 + costheta : 1.0 - costheta;
            double dcos[3][3];
            if (lgrad) {
              double df[3][3], dg[3][3];
              for (int c = 0; c < 3; c++) {
                df[0][c] = -2.0 * rij * drij[0][c] - 2.0 * rik * drik[0][c];
                df[1][c] = 2.0 * rjk * drjk[1][c] - 2.0 * rij * drij[1][c];
                df[2][c] = 2.0 * rjk * drjk[2][c] - 2.0 * rik * drik[2][c];
                dg[0][c] = -2.0 * (drij[0][c] * rik + rij * drik[0][c]);
                dg[1][c] = -2.0 * drij[1][c] * rik;
                dg[2][c] = -2.0 * rij * drik[2][c];
              }
              double tg = 1.0 / (g * g);
              for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                  if (type == 2)
                    dcos[r][c] = (df[r][c] * g - f * dg[r][c]) * tg;
                  else
                    dcos[r][c] = -1.0 * (df[r][c] * g - f * dg[r][c]) * tg;
                }
            }
            double expxyz = exp(-alpha * (rij * rij + rik * rik + rjk * rjk));
            /* angular factor: the reference's (1 +- cos) for zeta == 1 */
            double ang = costheta;
            double dang_scale = 1.0;
            if (zeta != 1.0) {
              double pref = pow(2.0, 1.0 - zeta);
              double base = costheta;
              ang = pref * pow(base, zeta);
              dang_scale = pref * zeta * pow(base, zeta - 1.0);
            }
            (void)lam;
            double val = ang * expxyz * fcutij * fcutik * fcutjk;
            XX(ii, i) = XX(ii, i) + val;
            XX(ii + nnn, i) = XX(ii + nnn, i) + ang * expxyz * fcutij * fcutik * fcutjk * wj * wk;
            if (!lgrad) continue;
            double dexp[3][3];
            double te = -alpha * 2.0 * expxyz;
            for (int r = 0; r < 3; r++)
              for (int c = 0; c < 3; c++)
                dexp[r][c] = (rij * drij[r][c] + rik * drik[r][c] + rjk * drjk[r][c]) * te;
            for (int c = 0; c < 3; c++) {
              double t[3], tw[3];
              for (int r = 0; r < 3; r++) {
                double dc = dcos[r][c] * dang_scale;
                t[r] = dc * expxyz * fcutij * fcutik * fcutjk
                     + ang * dexp[r][c] * fcutij * fcutik * fcutjk
                     + ang * expxyz * dfij[r][c] * fcutik * fcutjk
                     + ang * expxyz * fcutij * dfik[r][c] * fcutjk
                     + ang * expxyz * fcutij * fcutik * dfjk[r][c];
                tw[r] = t[r] * wj * wk;
              }
              DXDY(ii, i, i, c) = DXDY(ii, i, i, c) + t[0];
              DXDY(ii, i, n, c) = DXDY(ii, i, n, c) + t[1];
              DXDY(ii, i, mm, c) = DXDY(ii, i, mm, c) + t[2];
              DXDY(ii + nnn, i, i, c) = DXDY(ii + nnn, i, i, c) + tw[0];
              DXDY(ii + nnn, i, n, c) = DXDY(ii + nnn, i, n, c) + tw[1];
              DXDY(ii + nnn, i, mm, c) = DXDY(ii + nnn, i, mm, c) + tw[2];
              for (int a = 0; a < 3; a++) {
                STRS(a, c, ii, i) = STRS(a, c, ii, i) + dj[a] * t[1] + dk[a] * t[2];
                STRS(a, c, ii + nnn, i) = STRS(a, c, ii + nnn, i) + dj[a] * tw[1] + dk[a] * tw[2];
              }
            }
          }
        }
      }
    }
    /* any other type: the reference prints "Unknown function type" and
     * leaves the descriptor at zero (wacsf.f90:792-794) */
  }
#undef XX
#undef DXDY
#undef STRS
#undef NB
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* FGAP_CALC, gap_calc.f90:1-301                                             */
/* ------------------------------------------------------------------------ */
int orc_gap_calc(const orc_model *m, int na, const int *species,
                 const double *lat, const double *pos, double rcut, int lgrad,
                 double *ene, double *force, double *stress, double *variance,
                 double *xx_out, double *dedg_out, double *e_out) {
  const int D = m->des_len, M = m->nsparse;
  const int max_nb = 1000; /* gap_calc.f90:68 */
  int st = ORC_OK;
  double *weights = NULL, *nb = NULL, *xx = NULL, *dxdy = NULL, *strs = NULL;
  double *ckm = NULL, *e = NULL, *dedg = NULL;
  int *count = NULL;
  if (na <= 0) return ORC_ERR_ARG;

  /* gap_calc.f90:75-83 - an atom whose Z is not in the table keeps an
   * undefined weight in the reference; here it is an error. */
  weights = (double *)malloc(sizeof(double) * na);
  if (!weights) return ORC_ERR_ALLOC;
  for (int j = 0; j < na; j++) {
    int found = 0;
    for (int s = 0; s < m->nspecies; s++)
      if (species[j] == m->species_z[s]) { weights[j] = m->species_w[s]; found = 1; }
    if (!found) { free(weights); return ORC_ERR_UNKNOWN_SPECIES; }
  }

  count = (int *)malloc(sizeof(int) * na);
  nb = (double *)malloc(sizeof(double) * (size_t)na * max_nb * 6);
  xx = (double *)malloc(sizeof(double) * (size_t)na * D);
  if (!count || !nb || !xx) { st = ORC_ERR_ALLOC; goto out; }
  if (lgrad) {
    dxdy = (double *)malloc(sizeof(double) * (size_t)D * na * na * 3);
    strs = (double *)malloc(sizeof(double) * (size_t)9 * D * na);
    if (!dxdy || !strs) { st = ORC_ERR_ALLOC; goto out; }
  }
  st = orc_neighbors(na, lat, pos, weights, rcut, max_nb, count, nb);
  if (st) goto out;
  st = orc_car2acsf(m, na, max_nb, pos, nb, count, xx, dxdy, strs, lgrad);
  if (st) goto out;

  /* GET_COV, gap_calc.f90:143-147, 268-288 */
  ckm = (double *)malloc(sizeof(double) * (size_t)na * M);
  e = (double *)malloc(sizeof(double) * na);
  dedg = (double *)calloc((size_t)na * D, sizeof(double));
  if (!ckm || !e || !dedg) { st = ORC_ERR_ALLOC; goto out; }
  for (int i = 0; i < na; i++)
    for (int k = 0; k < M; k++) {
      double temp = 0.0;
      for (int d = 0; d < D; d++) {
        double q = (xx[(size_t)i * D + d] - m->mm[(size_t)k * D + d]) / m->theta[d];
        temp = temp + q * q;
      }
      ckm[(size_t)i * M + k] = ORC_DELTA * exp(-0.5 * temp);
    }
  /* gap_calc.f90:152-154 */
  double energy = 0.0;
  for (int i = 0; i < na; i++) {
    double s = 0.0;
    for (int k = 0; k < M; k++) s = s + ckm[(size_t)i * M + k] * m->coeff[k];
    e[i] = s;
  }
  for (int i = 0; i < na; i++) energy = energy + e[i];
  /* gap_calc.f90:157-166 */
  for (int i = 0; i < na; i++)
    for (int d = 0; d < D; d++) {
      double acc = 0.0;
      double th2 = m->theta[d] * m->theta[d];
      for (int k = 0; k < M; k++)
        acc = acc - 1.0 * (xx[(size_t)i * D + d] - m->mm[(size_t)k * D + d]) / th2
                        * ckm[(size_t)i * M + k] * m->coeff[k];
      dedg[(size_t)i * D + d] = acc;
    }
  *ene = energy;
  *variance = 0.0; /* gap_calc.f90:206 */
  for (int i = 0; i < na * 3; i++) force[i] = 0.0;
  for (int i = 0; i < 6; i++) stress[i] = 0.0;
  if (lgrad) {
    /* gap_calc.f90:177-185 */
    for (int i = 0; i < na; i++)
      for (int n = 0; n < na; n++)
        for (int c = 0; c < 3; c++) {
          double acc = force[i * 3 + c];
          const double *dx = dxdy + (((size_t)c * na + i) * na + n) * D;
          const double *dg = dedg + (size_t)n * D;
          for (int d = 0; d < D; d++) acc = acc - dg[d] * dx[d];
          force[i * 3 + c] = acc;
        }
    /* gap_calc.f90:189-203 */
    double sc[6];
    int k1 = 0;
    for (int a = 0; a < 3; a++)
      for (int b = a; b < 3; b++) {
        double acc = 0.0;
        for (int n = 0; n < na; n++)
          for (int d = 0; d < D; d++)
            acc = acc - dedg[(size_t)n * D + d] * strs[(((size_t)n * D + d) * 3 + b) * 3 + a];
        sc[k1++] = acc;
      }
    double vol = fabs(lat_det(lat));
    for (int q = 0; q < 6; q++) sc[q] = sc[q] * (1.0 / ORC_GPA2EVPANG) / vol;
    /* gap_calc.f90:221-226 */
    stress[0] = sc[0];
    stress[1] = sc[3];
    stress[2] = sc[5];
    stress[3] = sc[1];
    stress[4] = sc[4];
    stress[5] = sc[2];
  }
  if (xx_out) memcpy(xx_out, xx, sizeof(double) * (size_t)na * D);
  if (dedg_out) memcpy(dedg_out, dedg, sizeof(double) * (size_t)na * D);
  if (e_out) memcpy(e_out, e, sizeof(double) * na);
out:
  free(weights);
  free(count);
  free(nb);
  free(xx);
  free(dxdy);
  free(strs);
  free(ckm);
  free(e);
  free(dedg);
  return st;
}

int orc_gap_calc_batch(const orc_model *m, int nstruct, const int *atom_off,
                       const int *species, const double *lat,
                       const double *pos, double rcut, int nthreads,
                       double *ene, double *force, double *stress) {
  int st = ORC_OK;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int s = 0; s < nstruct; s++) {
    int a0 = atom_off[s], na = atom_off[s + 1] - atom_off[s];
    double var;
    int r = orc_gap_calc(m, na, species + a0, lat + (size_t)s * 9, pos + (size_t)a0 * 3,
                         rcut, 1, ene + s, force + (size_t)a0 * 3, stress + (size_t)s * 6,
                         &var, NULL, NULL, NULL);
    if (r) {
#ifdef _OPENMP
#pragma omp critical
#endif
      st = r;
    }
  }
  return st;
}

/* FGET_BOND, get_bond.f90:4-116 */
/* ------------------------------------------------------------------------ */
/* The predictive variance of the commented-out block of FGAP_CALC,
 * gap_calc.f90:206-210:
 *   covf(i)  = delta - dot_product(ckm(i,:), matmul(qmm, ckm(i,:)))
 *   VARIANCE = VARIANCE + covf(i)/na          (atom order)
 * with ckm from GET_COV (gap_calc.f90:268-288) on the descriptors xx[na][D].
 * qmm is [M][M] row-major, qmm[m*M+n] = qmm(m,n).  The reference zero-fills
 * qmm in FGAP_READ (gap_calc.f90:361) and returns VARIANCE = 0; this is the
 * formula it would evaluate for a caller-supplied qmm. */
int orc_variance(const orc_model *m, int na, const double *xx, const double *qmm,
                 double *covf, double *variance) {
  const int D = m->des_len, M = m->nsparse;
  if (na <= 0) return ORC_ERR_ARG;
  double *ck = (double *)malloc(sizeof(double) * M);
  double *tmp = (double *)malloc(sizeof(double) * M);
  if (!ck || !tmp) { free(ck); free(tmp); return ORC_ERR_ALLOC; }
  double var = 0.0;
  for (int i = 0; i < na; i++) {
    for (int k = 0; k < M; k++) {
      double temp = 0.0;
      for (int d = 0; d < D; d++) {
        double q = (xx[(size_t)i * D + d] - m->mm[(size_t)k * D + d]) / m->theta[d];
        temp = temp + q * q;
      }
      ck[k] = ORC_DELTA * exp(-0.5 * temp);
    }
    for (int a = 0; a < M; a++) {
      double s = 0.0;
      for (int b = 0; b < M; b++) s = s + qmm[(size_t)a * M + b] * ck[b];
      tmp[a] = s;
    }
    double dot = 0.0;
    for (int a = 0; a < M; a++) dot = dot + ck[a] * tmp[a];
    covf[i] = ORC_DELTA - dot;
    var = var + covf[i] / na;
  }
  *variance = var;
  free(ck);
  free(tmp);
  return ORC_OK;
}

double orc_min_bond(int na, const double *lat, const double *pos, double rcut) {
  int nabc[3];
  orc_nabc(lat, rcut, nabc);
  double min_bond = 10.0;
  for (int i = 0; i < na; i++)
    for (int j = 0; j < na; j++)
      for (int n1 = -nabc[0]; n1 <= nabc[0]; n1++)
        for (int n2 = -nabc[1]; n2 <= nabc[1]; n2++)
          for (int n3 = -nabc[2]; n3 <= nabc[2]; n3++) {
            if (n1 == 0 && n2 == 0 && n3 == 0 && i == j) continue;
            double dr[3];
            for (int c = 0; c < 3; c++) {
              double xyz = pos[j * 3 + c] + (double)n1 * lat[0 * 3 + c]
                         + (double)n2 * lat[1 * 3 + c] + (double)n3 * lat[2 * 3 + c];
              dr[c] = pos[i * 3 + c] - xyz;
            }
            double dis = sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
            if (dis > rcut) continue;
            if (dis < min_bond) min_bond = dis;
          }
  return min_bond;
}
