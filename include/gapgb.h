/*
 * gapgb.h - C ABI of the GB300 (sm_103a) CALYPSO-GAP energy / force / stress
 * evaluator: wACSF descriptors + sparse GPR, neighbour search, chain rule into
 * forces and virial stress, all on one GPU.
 *
 * Plain C types only (no CUDA or torch types); every call returns a status and
 * never exits the process.  Array conventions are C row-major as numpy callers
 * use them:
 *   lat[s*9 + a*3 + c]   row a = lattice vector a of structure s (Angstrom)
 *   pos[i*3 + c]         Cartesian position of atom i (Angstrom)
 *   force[i*3 + c]       eV/Angstrom
 *   stress[s*6 + q]      GPa, order XX YY ZZ XY YZ ZX, sign and units of the
 *                        reference (gappy/libgap/gap_calc.f90:201-226)
 * Ragged batches are packed: structure s owns atoms atom_off[s] ..
 * atom_off[s+1]-1 (atom_off has nstruct+1 entries, atom_off[0] == 0).
 *
 * A handle is not thread-safe: use one handle per host thread (the reference
 * itself is not re-entrant: it opens fixed Fortran units 111/2233/2244).
 */
#ifndef GAPGB_H
#define GAPGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GAPGB_OK = 0,
  GAPGB_ERR_FILE = 1,               /* model file missing / unreadable */
  GAPGB_ERR_PARSE = 2,              /* model file malformed */
  GAPGB_ERR_CAP_EXCEEDED = 3,       /* size beyond a documented limit */
  GAPGB_ERR_UNKNOWN_SPECIES = 4,    /* atomic number absent from the model */
  GAPGB_ERR_NEIGHBOUR_OVERFLOW = 5, /* more neighbours than the capacity */
  GAPGB_ERR_CUDA = 6,               /* CUDA runtime error (see gapgb_last_error) */
  GAPGB_ERR_TIMEOUT = 7,            /* a bounded device wait gave up */
  GAPGB_ERR_ARG = 8,                /* invalid argument */
  GAPGB_ERR_ALLOC = 9,              /* host or device allocation failed */
  GAPGB_ERR_NO_DEVICE = 10          /* no CUDA device visible */
} gapgb_status;

/* Arithmetic of the evaluation. */
typedef enum {
  GAPGB_PREC_FP64 = 0, /* plain path: FP64 everywhere, matches the reference */
  GAPGB_PREC_FP32 = 1, /* FP32 descriptors and GPR, FP64 energy/virial sums */
  GAPGB_PREC_TC = 2,   /* FP32 descriptors, tensor-core GPR (split BF16, FP32
                          accumulate), FP64 energy/virial sums */
  GAPGB_PREC_MIXED = 3, /* FP32 descriptors and gradients, FP64 GPR (for models
                          whose coefficients cancel strongly) */
  GAPGB_PREC_SURROGATE = 4, /* FP32 descriptors, the attached learned surrogate
                              for e and dE/dG, FP64 GPR (the mixed form) for
                              the atoms whose committee disagrees; needs
                              gapgb_model_set_surrogate first */
  GAPGB_PREC_TF32 = 5      /* FP32 descriptors, tensor-core GPR with single
                              TF32 products and FP32 accumulation; D <= 64 */
} gapgb_precision;
/* In the forms other than FP64, the fast descriptor-gradient kernel (taken
 * when every angular SF shares one cutoff, up to 4 angular alphas and 8
 * (lambda, zeta) combinations) sums each neighbour slot's gradient in fixed
 * point: every pair term is rounded to 2^-29 eV/A, and a term beyond 2047
 * eV/A or not finite makes the call return GAPGB_ERR_CAP_EXCEEDED (the FP64
 * form has no such limit).  These slot sums do not depend on the order of
 * the device's atomic adds. */

typedef enum {
  GAPGB_OPT_PRECISION = 0,     /* gapgb_precision, default GAPGB_PREC_FP64 */
  GAPGB_OPT_NEIGHBOUR_CAP = 1, /* slots per atom, default 256; grown on overflow
                                  by the host-buffer calls */
  GAPGB_OPT_DEVICE = 2,        /* CUDA device ordinal, default 0 */
  GAPGB_OPT_GENERIC_KERNELS = 3, /* 1: FP32 descriptor kernels take the generic
                                    path even when the fast path applies */
  GAPGB_OPT_PIPELINES = 4        /* 1 or 2 (default 2): a batch of at least
                                    20480 atoms in the TC / TF32 forms (grouped
                                    descriptor kernels, gradients on) is
                                    evaluated as two halves on two streams, so
                                    one half's kernels fill the SMs the other
                                    half's leave idle; results are the same */
} gapgb_option;

typedef struct gapgb_model gapgb_model;

const char *gapgb_status_string(gapgb_status st);
/* Text of the last error seen on this host thread ("" if none). */
const char *gapgb_last_error(void);
/* Library version string. */
const char *gapgb_version(void);

/* ---- model ------------------------------------------------------------ */

/* Parse a gap_parameters file and upload it to the device.
 * Replaces FGAP_READ (gappy/libgap/gap_calc.f90:303-364) together with the
 * species-weight read of FGAP_CALC (gap_calc.f90:75-83) and the SF-table read
 * of CAR2ACSF (gappy/libgap/wacsf.f90:40-56).  rcut is the neighbour cutoff
 * the reference passes to FGAP_CALC (gappy/libgap/GAP.py:15, default 6.0).
 * Unlike the reference, M > 4000 and D > 100 are accepted. */
gapgb_status gapgb_model_load(const char *path, double rcut, gapgb_model **out);

/* Build a model from arrays (same meaning as the file's blocks).
 * sf_zeta may be NULL (all 1, the reference's angular exponent);
 * mm is [nsparse * des_len] row-major (row k = sparse point k). */
gapgb_status gapgb_model_create(int nspecies, const int *species_z,
                                const double *species_w, int nsf,
                                const int *sf_type, const double *sf_alpha,
                                const double *sf_cutoff, const double *sf_zeta,
                                int nsparse, int des_len, const double *theta,
                                const double *mm, const double *coeff,
                                double rcut, gapgb_model **out);

/* Write the model as a gap_parameters file (the grammar FGAP_READ and
 * CAR2ACSF read, gap_calc.f90:303-364 and wacsf.f90:45-56): the species
 * and SF tables, "M D", three blank records, theta, one record per sparse
 * point, coeff.  Values are written with 17 significant digits, so
 * gapgb_model_load gives back the same arrays; the zeta column appears only
 * where zeta != 1.  With gapgb_model_create this is the writer a fitting
 * code uses to hand a new model to the reference's readers. */
gapgb_status gapgb_model_write(const gapgb_model *model, const char *path);

void gapgb_model_free(gapgb_model *model);

gapgb_status gapgb_model_info(const gapgb_model *model, int *nsparse,
                              int *des_len, int *nsf, int *nspecies,
                              double *rcut);

/* Host copies of theta[D], mm[M*D] (row-major), coeff[M]; any may be NULL. */
gapgb_status gapgb_model_arrays(const gapgb_model *model, double *theta,
                                double *mm, double *coeff);

/* Host copies of the species table (nspecies entries) and the SF table
 * (nsf entries); any pointer may be NULL.  With gapgb_model_create this
 * rebuilds a model from a file's tables and caller-supplied GPR arrays, as
 * FGAP_CALC does (gap_calc.f90:1-46 takes theta/MM/coeff as arguments and
 * reads the tables from ./gap_parameters). */
gapgb_status gapgb_model_tables(const gapgb_model *model, int *species_z,
                                double *species_w, int *sf_type,
                                double *sf_alpha, double *sf_cutoff,
                                double *sf_zeta);

gapgb_status gapgb_set_option(gapgb_model *model, gapgb_option opt,
                              int64_t value);
gapgb_status gapgb_get_option(const gapgb_model *model, gapgb_option opt,
                              int64_t *value);

/* ---- fitting ------------------------------------------------------------ */

/* Replace the model's coefficients c[M] (host and device copies). */
gapgb_status gapgb_model_set_coeff(gapgb_model *model, const double *coeff);

/* Fit c from training energies, on the device, and set it on the model.
 * The reference only evaluates E = sum_i sum_k c_k K(x_i, m_k)
 * (gap_calc.f90:143-154); its fitting codes are not part of the repository.
 * Sparse (subset-of-regressors) normal equations in FP64:
 *   Phi_sk = sum_{i in s} K(x_i, m_k)
 *   (K_MM + jitter I + sum_s w_s Phi_s^T Phi_s) c = sum_s w_s Phi_s^T E_s
 *   w_s = 1 / (sigma_e^2 n_s)   (sigma_e: energy noise per atom, eV)
 * solved by a blocked Cholesky factorisation.  Descriptors are the FP64
 * path's; the sparse points and theta are the model's.  energy[nstruct]
 * in eV; coeff[M] (may be NULL) receives c.  A matrix that is not positive
 * definite gives GAPGB_ERR_ARG (raise jitter). */
gapgb_status gapgb_fit_energies(gapgb_model *model, int nstruct,
                                const int *atom_off, const int *species,
                                const double *lat, const double *pos,
                                const double *energy, double sigma_e,
                                double jitter, double *coeff);

/* gapgb_fit_energies with force and stress rows as well: forces[natoms*3]
 * (eV/A) and stress[nstruct*6] (GPa, XX YY ZZ XY YZ ZX as gapgb_eval
 * reports it), either may be NULL, fitted with noise sigma_f (eV/A) and
 * sigma_s (GPa) per component,
 *   (K_MM + jitter I + sum_s w_s Phi_s^T Phi_s + PhiF^T PhiF / sigma_f^2
 *      + PhiS^T PhiS / sigma_s^2) c
 *       = sum_s w_s Phi_s^T E_s + PhiF^T F / sigma_f^2 + PhiS^T sigma / sigma_s^2,
 * where column k of PhiF / PhiS is the force field / stress of the model
 * with c = e_k (the FP64 chain rule run once per sparse point: meant for
 * training sets of the usual GAP size, hundreds of cells). */
gapgb_status gapgb_fit(gapgb_model *model, int nstruct, const int *atom_off,
                       const int *species, const double *lat,
                       const double *pos, const double *energy,
                       const double *forces, const double *stress,
                       double sigma_e, double sigma_f, double sigma_s,
                       double jitter, double *coeff);

/* ---- predictive variance ------------------------------------------------ */

/* Attach qmm, the nsparse x nsparse matrix of the reference's variance block
 * (FGAP_CALC's qmm argument, gap_calc.f90:40; the block itself,
 * gap_calc.f90:206-210, is commented out there and FGAP_READ zero-fills
 * qmm, so the reference always reports 0).  qmm is row-major,
 * qmm[m * nsparse + n] = qmm(m, n), copied; NULL detaches it.  nsparse must
 * equal the model's M. */
gapgb_status gapgb_model_set_qmm(gapgb_model *model, const double *qmm,
                                 int nsparse);

/* The variance block for a packed batch (host buffers):
 *   covf_i = delta - k_i^T qmm k_i,  k_i = GET_COV row of atom i, delta = 1
 *   variance[s] = mean of covf over structure s's atoms
 * covf [natoms] may be NULL.  FP64 and MIXED models compute K and the
 * N x M x M contraction in FP64; the other forms use FP32 K and tcgen05
 * split-BF16 products with FP32 accumulation.  Needs an attached qmm. */
gapgb_status gapgb_variance(gapgb_model *model, int nstruct,
                            const int *atom_off, const int *species,
                            const double *lat, const double *pos,
                            double *covf, double *variance);

/* Device time (ms) of the variance kernels of the last gapgb_variance call
 * (K, contraction, sums; not the neighbour list and descriptors).  Only
 * filled when GAPGB_PROFILE_STAGES is set in the environment. */
gapgb_status gapgb_variance_time(gapgb_model *model, float *ms);

/* ---- evaluation, host buffers ------------------------------------------- */

/* One structure.  Replaces FGAP_CALC (gappy/libgap/gap_calc.f90:1-301):
 * same inputs (species as atomic numbers, lattice rows, Cartesian
 * positions), same outputs (energy eV, forces eV/A, stress GPa in the order
 * XX YY ZZ XY YZ ZX, variance = 0 as in gap_calc.f90:206).  With lgrad == 0
 * force and stress are set to zero, as the reference leaves them.  When a
 * qmm is attached (gapgb_model_set_qmm) and variance is not NULL, variance
 * is the mean covf of gapgb_variance instead. */
gapgb_status gapgb_eval(gapgb_model *model, int natoms, const int *species,
                        const double *lat, const double *pos, int lgrad,
                        double *energy, double *force, double *stress,
                        double *variance);

/* A packed ragged batch of independent structures in one pass (the batched
 * replacement for one FGAP_CALC call per structure).  Host buffers; pinned
 * host memory makes the copies asynchronous.  atom_energy may be NULL. */
gapgb_status gapgb_eval_batch(gapgb_model *model, int nstruct,
                              const int *atom_off, const int *species,
                              const double *lat, const double *pos, int lgrad,
                              double *energy, double *force, double *stress,
                              double *atom_energy);

/* ---- evaluation, device buffers ----------------------------------------- */

/* Same as gapgb_eval_batch with every array in device memory, enqueued on
 * `stream` (a cudaStream_t, NULL = legacy default stream) without a host
 * synchronisation, so the call can be captured in a CUDA graph.  natoms must
 * equal atom_off[nstruct] and max_atoms must bound every structure's atom
 * count.  Errors found on the device (neighbour overflow, unknown species)
 * are reported by gapgb_check_device_status after the stream has finished. */
gapgb_status gapgb_eval_batch_device(gapgb_model *model, int nstruct,
                                     int natoms, int max_atoms,
                                     const int *d_atom_off,
                                     const int *d_species, const double *d_lat,
                                     const double *d_pos, int lgrad,
                                     double *d_energy, double *d_force,
                                     double *d_stress, double *d_atom_energy,
                                     void *stream);

/* Reads and clears the device-side error flags of the last device-buffer
 * evaluation (synchronises the model's device). */
gapgb_status gapgb_check_device_status(gapgb_model *model);

/* A device-buffer evaluation captured once into a CUDA graph and replayed.
 * gapgb_graph_create runs one warm-up evaluation (which sizes the workspace,
 * builds the tensor-core image and checks the device flags), then captures
 * the same launch sequence; the graph stays bound to these buffers, so the
 * caller refills d_pos / d_lat (same sizes) between launches.  Structure
 * search evaluates a whole ragged population with one graph launch; MD
 * replays it every step.  While a graph (or an MD object) built from a model
 * is alive, the model refuses with GAPGB_ERR_ARG what would move the buffers
 * the graph captured: gapgb_set_option, gapgb_model_set_surrogate, and any
 * host-buffer call larger than the workspace the graph was built with.
 * gapgb_model_set_coeff is allowed: the tensor-core operand images are
 * rewritten in place and the graph replays with the new coefficients. */
typedef struct gapgb_graph gapgb_graph;
gapgb_status gapgb_graph_create(gapgb_model *model, int nstruct, int natoms,
                                int max_atoms, const int *d_atom_off,
                                const int *d_species, const double *d_lat,
                                const double *d_pos, int lgrad,
                                double *d_energy, double *d_force,
                                double *d_stress, double *d_atom_energy,
                                gapgb_graph **out);
gapgb_status gapgb_graph_launch(gapgb_graph *graph, void *stream);
void gapgb_graph_free(gapgb_graph *graph);

/* Device time of each stage of the last evaluation, in milliseconds:
 * t[0] neighbours, t[1] descriptors, t[2] GPR, t[3] chain rule + reduction.
 * Only filled when GAPGB_PROFILE_STAGES is set in the environment. */
gapgb_status gapgb_stage_times(gapgb_model *model, float t[4]);

/* Measured arithmetic peaks of the current device, the roofline denominators
 * of the SIMT kernels (no counterpart in the reference, which has no device
 * code): out[0] FP32 FMA TFLOP/s, out[1] FP64 FMA TFLOP/s (an FMA = 2 flops),
 * out[2] MUFU ex2 rate in 1e12 per second.  Each is one kernel of
 * independent FMA / ex2 chains on every SM (one resident wave), timed by
 * CUDA events after a warm-up launch (well under a second in all). */
gapgb_status gapgb_measure_peaks(double out[3]);

/* ---- GPR step without device allocation ---------------------------------- */

/* Atomic energies e[natoms] and dE/dG[natoms*D] (FP64, row-major) from FP64
 * descriptors d_G[natoms*D] already in device memory, enqueued on `stream`
 * with no device allocation of any kind.  No counterpart in the reference:
 * it serves callers that cannot allocate when they need the GPR - hosts
 * (simulation engines, serving processes) that reserve all device memory up
 * front in their own pool, where a cudaMalloc behind their back fails or
 * eats into the pool, and loops that cannot take the device-wide
 * synchronisation cudaMalloc / cudaFree may cause.
 * Working memory is one fixed 8 MiB array in device memory per GPU, held
 * until the process exits; calls with natoms * (D + 1) > 1048576 (16131 atoms
 * at D = 64) return GAPGB_ERR_CAP_EXCEEDED.  The model must already be
 * resident on the device (any evaluation uploads it; this call never does).
 * The first call on a device also does a one-time set-up (the array's device
 * address, the kernel's shared-memory limit).  All calls share the array:
 * calls that overlap on the GPU (other streams, other host threads) race and
 * must be serialised by the caller, and every call must have finished before
 * gapgb_model_set_coeff rewrites the coefficients it reads. */
gapgb_status gapgb_gpr_noalloc(gapgb_model *model, int natoms,
                               const double *d_G, double *d_e, double *d_dedg,
                               void *stream);

/* ---- learned surrogate with GPR fallback --------------------------------- */

/* No counterpart in the reference, which evaluates the GPR only.  A committee
 * of `members` per-species networks D -> H -> H -> 1 (SiLU) maps a descriptor
 * to an atomic energy; its input gradient replaces dE/dG, so forces and
 * stress follow through the same chain rule.  Trained on the GAP's own
 * atomic energies and dE/dG (per atom: forces are the fixed linear map
 * F = -J^T dE/dG of them) with the library's own forward, backward and Adam
 * kernels: BF16 weights and row operands, FP32 accumulation, FP32 master
 * weights.  In an evaluation at GAPGB_PREC_SURROGATE, atoms whose committee
 * standard deviation exceeds the threshold take the exact GPR instead. */
typedef struct gapgb_surrogate gapgb_surrogate;

/* Random initialisation from `seed` on the current CUDA device. */
gapgb_status gapgb_surrogate_create(int nspecies, const int *species_z,
                                    int des_len, int hidden, int members,
                                    unsigned long long seed,
                                    gapgb_surrogate **out);
void gapgb_surrogate_free(gapgb_surrogate *s);
gapgb_status gapgb_surrogate_info(const gapgb_surrogate *s, int *nspecies,
                                  int *des_len, int *hidden, int *members,
                                  size_t *params_per_block);

/* Input standardisation (mean, std per descriptor component; components with
 * std <= 1e-12 pass through) and the energy normalisation e = e_scale * y +
 * e_shift[species]. */
gapgb_status gapgb_surrogate_set_norm(gapgb_surrogate *s, const double *g_mean,
                                      const double *g_std,
                                      const double *e_shift, double e_scale);

/* FP32 master weights, members * nspecies blocks of params_per_block floats
 * in the order block (q * nspecies + s) = {W1[H][D], b1[H], W2[H][H], b2[H],
 * w3[H], b3, zeros}: params_per_block is rounded up to a multiple of 8 and the
 * tail stays zero.  `get` copies them out, `set` replaces them (and resets
 * Adam); either may be NULL. */
gapgb_status gapgb_surrogate_params(gapgb_surrogate *s, float *get,
                                    const float *set);

/* One training step of every (member, species) block at once.  d_rows holds
 * members * nspecies * rows_per_species atom indices (device; block order as
 * above, each block's rows of that species) into the label arrays: FP32
 * descriptors d_G[n*D], atomic energies d_e[n] (eV), dE/dG d_dedg[n*D].
 * rows_per_species is a multiple of 64.  Loss per block: mean over its rows
 * of (y - y*)^2 + lambda |dy/dx - t*|^2 in normalised units.  With update,
 * one Adam step (lr, beta 0.9 / 0.999, eps 1e-8).  loss (host, nullable)
 * receives the members * nspecies block losses (this call then waits for the
 * step); d_grad (device, nullable) the weight gradient in the params layout.
 * The step runs on the surrogate's own stream: the caller makes d_rows and
 * the labels complete on the device before the call. */
gapgb_status gapgb_surrogate_train_step(gapgb_surrogate *s, int rows_per_species,
                                        const int *d_rows, const float *d_G,
                                        const double *d_e, const float *d_dedg,
                                        float lambda, float lr, int update,
                                        double *loss, float *d_grad);

/* Committee prediction for natoms atoms (atomic numbers d_species, FP32
 * descriptors d_G, device): mean atomic energy d_e (eV), committee standard
 * deviation d_std (eV), mean dE/dG d_dedg[natoms*D] and, when d_gstd is not
 * NULL, the members' dE/dG spread per atom (as gapgb_model_set_fallback_
 * triggers reads it).  Waits for the stream (NULL: the surrogate's own
 * stream). */
gapgb_status gapgb_surrogate_predict(gapgb_surrogate *s, int natoms,
                                     const int *d_species, const float *d_G,
                                     double *d_e, float *d_std, float *d_dedg,
                                     float *d_gstd, void *stream);

/* Attach a surrogate (not owned; NULL detaches) and the fallback threshold
 * on the committee standard deviation, in eV.  Its des_len must be the
 * model's D and its species must include every species of the model.
 * Detaching while the precision is GAPGB_PREC_SURROGATE sets it to
 * GAPGB_PREC_MIXED. */
gapgb_status gapgb_model_set_surrogate(gapgb_model *model, gapgb_surrogate *s,
                                       double threshold_ev);

/* Force-sensitive fallback triggers of the surrogate form (no counterpart in
 * the reference).  At GAPGB_PREC_SURROGATE an atom also takes the exact GPR,
 * whatever its energy-committee spread, when
 *  - the committee members' dE/dG vectors spread by more than grad_spread
 *    (the norm over the D components of their standard deviation, eV per
 *    descriptor unit): a force error comes from a dE/dG error, which the
 *    energy spread does not see; or
 *  - any of its neighbours is closer than r_contact (Angstrom): at short
 *    contacts the descriptor Jacobian amplifies a small dE/dG error into a
 *    large force error; both atoms of such a contact see it.
 * 0 (the default) turns a trigger off.  Refused while a graph of the model
 * lives. */
gapgb_status gapgb_model_set_fallback_triggers(gapgb_model *model, double grad_spread,
                                               double r_contact);

/* Number of atoms that took the GPR fallback in the model's last
 * GAPGB_PREC_SURROGATE evaluation (synchronises the model's device). */
gapgb_status gapgb_surrogate_fallback_count(gapgb_model *model, int *count);

/* Training labels: FP32 descriptors d_G[n*D], atomic energies d_e[n] and
 * dE/dG d_dedg[n*D] (device) of a packed batch (host inputs as in
 * gapgb_eval_batch), from the model's GPR at its current precision (any but
 * GAPGB_PREC_SURROGATE). */
gapgb_status gapgb_gpr_labels(gapgb_model *model, int nstruct,
                              const int *atom_off, const int *species,
                              const double *lat, const double *pos,
                              float *d_G, double *d_e, float *d_dedg);

/* ---- molecular dynamics --------------------------------------------------- */

/* NVE velocity-Verlet MD of a packed batch of fixed cells on the device.  No
 * counterpart in the reference's hot path: gappy runs MD through ASE with
 * one FGAP_CALC per step (gappy/example/ASE-GAPPY/run_md.py:10-27).  Units:
 * Angstrom, fs, amu (d_mass[natoms]), eV; d_pos[natoms*3] and d_vel[natoms*3]
 * (Angstrom/fs) are device arrays the object advances in place.  The
 * neighbour list is built with cutoff rcut + skin every rebuild_every steps
 * (atoms wrapped into their cells first) and refreshed from the current
 * positions in between; slots beyond the cutoff contribute exactly zero, so
 * a refreshed step equals a fresh build up to summation order.  An atom that
 * moves more than skin/2 between rebuilds is reported by gapgb_md_check.
 * Each step is one CUDA graph launch.  gapgb_md_create evaluates the forces
 * at t = 0 (growing the neighbour capacity with 25 % headroom) and captures
 * the two step graphs; the model is dedicated to the MD object while it
 * lives (its workspace holds the list) and must not be reconfigured. */
typedef struct gapgb_md gapgb_md;
gapgb_status gapgb_md_create(gapgb_model *model, int nstruct, int natoms,
                             const int *d_atom_off, const int *d_species,
                             const double *d_lat, double *d_pos, double *d_vel,
                             const double *d_mass, double dt_fs, double skin,
                             int rebuild_every, gapgb_md **out);
/* nsteps steps on `stream` (NULL: the object's stream); per step, the
 * potential energy of each structure is appended to d_epot[k*nstruct + s]
 * and the kinetic energy to d_ekin (device, either may be NULL). */
gapgb_status gapgb_md_run(gapgb_md *md, int nsteps, double *d_epot,
                          double *d_ekin, void *stream);
/* Device pointers of the latest step's energy[nstruct], force[natoms*3],
 * stress[nstruct*6] (GPa, reference order) and kinetic energy[nstruct]. */
gapgb_status gapgb_md_outputs(const gapgb_md *md, const double **d_energy,
                              const double **d_force, const double **d_stress,
                              const double **d_ekin);
/* Synchronises and reports the device flags raised since the last check
 * (neighbour overflow, skin exceeded, unknown species). */
gapgb_status gapgb_md_check(gapgb_md *md);
void gapgb_md_free(gapgb_md *md);

/* ---- descriptor export and utilities ------------------------------------ */

/* wACSF descriptors XX (D per atom, the reference layout of
 * gappy/libgap/wacsf.f90:86-87: unweighted block then weighted block) for a
 * packed batch; the working replacement for gappy/libgap/WACSF.py:43-52. */
gapgb_status gapgb_descriptors(gapgb_model *model, int nstruct,
                               const int *atom_off, const int *species,
                               const double *lat, const double *pos,
                               double *xx);

/* Neighbour list of one structure in the reference order (j, then n1, n2, n3
 * ascending; gappy/libgap/gap_calc.f90:92-120).  Writes count[natoms] and, for
 * slot q of atom i (q < count[i] <= cap), nb[(i*cap+q)*6 + f] with
 * f = 0..2 image xyz, 3 r, 4 weight of j, 5 j (1-based) - the reference's
 * neighbor(i, q, 1:6).  Distances are bit-identical to the reference loop
 * evaluated without fused multiply-adds. */
gapgb_status gapgb_neighbors(gapgb_model *model, int natoms,
                             const int *species, const double *lat,
                             const double *pos, int cap, int *count,
                             double *nb);

/* Minimum interatomic distance within rcut over all periodic images, 10.0 if
 * none; replaces FGET_BOND (gappy/libgap/get_bond.f90:4-116). */
gapgb_status gapgb_min_bond(int natoms, const double *lat, const double *pos,
                            double rcut, double *min_bond);

#ifdef __cplusplus
}
#endif
#endif /* GAPGB_H */
