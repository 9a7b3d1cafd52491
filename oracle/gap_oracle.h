/*
 * gap_oracle.h - CPU FP64 restatement of CALYPSO-GAP's energy/force/stress
 * evaluation (gappy/libgap/gap_calc.f90, gappy/libgap/wacsf.f90,
 * gappy/libgap/get_bond.f90).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle that the CUDA
 * product path is compared against, and the CPU baseline that bench.py times.
 * The product library never links, loads or calls it.
 *
 * Layout conventions (C row-major, matching numpy callers):
 *   lat[a*3+c]   row a = lattice vector a (the reference's LAT(a,:))
 *   pos[i*3+c]   Cartesian position of atom i (the reference's POS(i,:))
 *   force[i*3+c] force on atom i
 *   stress[6]    GPa, order XX YY ZZ XY YZ ZX (gap_calc.f90:221-226)
 *   xx[i*D+d]    descriptor d of atom i (the reference's XX(d,i))
 *   dedg[i*D+d]  dE/dG (gap_calc.f90:157-166)
 *   nb[(i*max_nb+k)*6 + f]  neighbour k of atom i: f=0..2 image xyz, 3 r,
 *                           4 weight of j, 5 j (1-based, as in the reference)
 */
#ifndef GAP_ORACLE_H
#define GAP_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_OK = 0,
  ORC_ERR_FILE = 1,
  ORC_ERR_PARSE = 2,
  ORC_ERR_CAP = 3,
  ORC_ERR_UNKNOWN_SPECIES = 4,
  ORC_ERR_NEIGHBOUR_OVERFLOW = 5,
  ORC_ERR_ALLOC = 6,
  ORC_ERR_ARG = 7
};

typedef struct {
  int nspecies;
  int species_z[128];
  double species_w[128];
  int nsf;
  int sf_type[256];
  double sf_alpha[256];
  double sf_cutoff[256];
  double sf_zeta[256]; /* optional 4th column of angular SF lines; 1 if absent */
  int nsparse;         /* M */
  int des_len;         /* D */
  double *theta;       /* [D] */
  double *mm;          /* [M*D], mm[k*D+d] */
  double *coeff;       /* [M] */
} orc_model;

int orc_model_read(const char *path, orc_model *m);
void orc_model_free(orc_model *m);

/* gap_calc.f90:85-88: images per lattice direction. */
void orc_nabc(const double *lat, double rcut, int nabc[3]);

/* gap_calc.f90:89-120: neighbour enumeration in the reference order. */
int orc_neighbors(int na, const double *lat, const double *pos,
                  const double *weights, double rcut, int max_nb,
                  int *count, double *nb);

/* wacsf.f90:2-796: descriptors (and, if dxdy/strs are non-NULL and lgrad,
 * the dense Jacobian dxdy[((c*na+j)*na+i)*D+d] = XX(d,i) / d pos(j,c)
 * and strs[((i*D+d)*3+b)*3+a] = STRS(a,b,d,i)). */
int orc_car2acsf(const orc_model *m, int na, int max_nb, const double *pos,
                 const double *nb, const int *count, double *xx,
                 double *dxdy, double *strs, int lgrad);

/* gap_calc.f90:1-301: the whole FGAP_CALC.  Optional outputs may be NULL:
 * xx_out[na*D], dedg_out[na*D], e_out[na] (atomic energies). */
int orc_gap_calc(const orc_model *m, int na, const int *species,
                 const double *lat, const double *pos, double rcut, int lgrad,
                 double *ene, double *force, double *stress, double *variance,
                 double *xx_out, double *dedg_out, double *e_out);

/* Many independent structures (packed: atom_off[s]..atom_off[s+1]) on
 * nthreads host threads, one structure per thread at a time - the way
 * structure-search callers farm the single-threaded reference. */
int orc_gap_calc_batch(const orc_model *m, int nstruct, const int *atom_off,
                       const int *species, const double *lat,
                       const double *pos, double rcut, int nthreads,
                       double *ene, double *force, double *stress);

/* get_bond.f90:4-116: minimum image distance within rcut (10.0 if none). */
/* gap_calc.f90:206-210 (commented out in the reference): per-atom
 * covf = delta - k^T qmm k and their mean, from descriptors xx[na][D]. */
int orc_variance(const orc_model *m, int na, const double *xx, const double *qmm,
                 double *covf, double *variance);
double orc_min_bond(int na, const double *lat, const double *pos, double rcut);

#ifdef __cplusplus
}
#endif
#endif
