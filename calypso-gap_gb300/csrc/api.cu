// api.cu - the C ABI (include/gapgb.h): models, workspace, evaluation.
//
// One evaluation of a packed batch is, in stream order:
//   prep (lattice images, weights)  -> neighbour list
//   -> descriptors G -> GPR (e, dE/dG) -> slot gradients + per-atom virial
//   -> forces -> per-structure energy and stress.
// The grouped FP32 gradient kernel scatters the forces itself; the FP64 path
// and the generic FP32 kernels add reverse slots after the neighbour list and
// gather the forces (deterministic).  This is FGAP_CALC
// (gappy/libgap/gap_calc.f90:1-301) for many structures at once, without the
// dense Jacobian.  The host-buffer calls synchronise once: the descriptor
// kernels take the previous call's slot count, and a batch that needs more
// slots or overflows the neighbour capacity is recomputed after a sync that
// sizes shared memory and grows the capacity.  The device-buffer call never
// synchronises.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <mutex>

#include "gapgb_internal.h"

namespace gapgb {

static thread_local std::string g_last_error;

void set_last_error(const std::string &s) { g_last_error = s; }

namespace {

gapgb_status fail(gapgb_status st, const std::string &msg) {
  set_last_error(msg);
  return st;
}

template <typename T>
void free_dev(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

void free_ws(Workspace &ws) {
  free_dev(ws.d_atom_off);
  free_dev(ws.d_species);
  free_dev(ws.d_lat);
  free_dev(ws.d_pos);
  free_dev(ws.d_energy);
  free_dev(ws.d_force);
  free_dev(ws.d_stress);
  free_dev(ws.d_atom_e);
  free_dev(ws.apos);
  free_dev(ws.frac32);
  free_dev(ws.pos2f);
  free_dev(ws.atom_struct);
  free_dev(ws.sinfo);
  free_dev(ws.nbr_cnt);
  free_dev(ws.nbr_j);
  free_dev(ws.nbr_s);
  free_dev(ws.nbr_rev);
  free_dev(ws.nbr_xyz);
  free_dev(ws.nbr_d32);
  free_dev(ws.nbr_w32);
  free_dev(ws.G);
  free_dev(ws.dedg);
  free_dev(ws.gslot);
  free_dev(ws.e);
  free_dev(ws.wvir);
  free_dev(ws.red_part);
  free_dev(ws.bin_count);
  free_dev(ws.bin_start);
  free_dev(ws.bin_atoms);
  free_dev(ws.atom_bin);
  free_dev(ws.atom_slot);
  free_dev(ws.atom_m);
  free_dev(ws.pairs);
  free_dev(ws.pair_cnt);
  free_dev(ws.d_flags);
  free_dev(ws.orphans);
  free_dev(ws.gpr_scratch);
  free_dev(ws.tc_scratch);
  ws.tc_scratch_size = 0;
  if (ws.h_flags) cudaFreeHost(ws.h_flags);
  ws.h_flags = nullptr;
  ws.N = ws.S = ws.cap = ws.D = 0;
  ws.gpr_scratch_size = 0;
}

#define WS_ALLOC(ptr, count)                                                        \
  do {                                                                              \
    if (cudaMalloc((void **)&(ptr), sizeof(*(ptr)) * (size_t)(count) + 16) !=       \
        cudaSuccess) {                                                              \
      free_ws(ws);                                                                  \
      return fail(GAPGB_ERR_ALLOC, "cudaMalloc failed for workspace");              \
    }                                                                               \
  } while (0)

gapgb_status ensure_ws(gapgb_model *m, int N, int S, int cap) {
  Workspace &ws = m->ws;
  const int D = m->host.D;
  const size_t scratch = gpr_scratch_bytes(N, m->host.M, D, sizeof(double));
  if (ws.d_flags && N <= ws.N && S <= ws.S && cap <= ws.cap && D == ws.D &&
      scratch <= ws.gpr_scratch_size)
    return GAPGB_OK;
  if (m->live_graphs->load() > 0)
    return fail(GAPGB_ERR_ARG,
                "the workspace would move while a CUDA graph built from this model is alive "
                "(free the graph first, or create it for the largest batch)");
  // grow with headroom so that slightly larger batches do not reallocate
  int nN = N > ws.N ? N + N / 8 : ws.N;
  int nS = S > ws.S ? S + S / 8 : ws.S;
  int nC = cap > ws.cap ? cap : ws.cap;
  free_ws(ws);
  const size_t nslots = (size_t)nN * nC;
  WS_ALLOC(ws.d_atom_off, nS + 1);
  WS_ALLOC(ws.d_species, nN);
  WS_ALLOC(ws.d_lat, (size_t)nS * 9);
  WS_ALLOC(ws.d_pos, (size_t)nN * 3);
  WS_ALLOC(ws.d_energy, nS);
  WS_ALLOC(ws.d_force, (size_t)nN * 3);
  WS_ALLOC(ws.d_stress, (size_t)nS * 6);
  WS_ALLOC(ws.d_atom_e, nN);
  WS_ALLOC(ws.apos, nN);
  WS_ALLOC(ws.frac32, nN);
  WS_ALLOC(ws.pos2f, (size_t)nN * 2);
  WS_ALLOC(ws.atom_struct, nN);
  WS_ALLOC(ws.sinfo, nS);
  WS_ALLOC(ws.nbr_cnt, nN);
  WS_ALLOC(ws.nbr_j, nslots);
  WS_ALLOC(ws.nbr_s, nslots);
  WS_ALLOC(ws.nbr_rev, nslots);
  WS_ALLOC(ws.nbr_xyz, nslots);
  WS_ALLOC(ws.nbr_d32, nslots);
  WS_ALLOC(ws.nbr_w32, nslots);
  WS_ALLOC(*(double **)&ws.G, (size_t)nN * D);
  WS_ALLOC(*(double **)&ws.dedg, (size_t)nN * D);
  WS_ALLOC(*(double4 **)&ws.gslot, nslots);
  WS_ALLOC(ws.e, nN);
  WS_ALLOC(ws.wvir, (size_t)nN * 9);
  WS_ALLOC(ws.red_part, (size_t)nS * 64 * 7);
  WS_ALLOC(ws.bin_count, (size_t)nN + 1);
  WS_ALLOC(ws.bin_start, (size_t)nN + 2);
  WS_ALLOC(ws.bin_atoms, nN);
  WS_ALLOC(ws.atom_bin, nN);
  WS_ALLOC(ws.atom_slot, nN);
  WS_ALLOC(ws.atom_m, nN);
  WS_ALLOC(ws.pairs, (size_t)nN * kPairCap);
  WS_ALLOC(ws.pair_cnt, nN);
  WS_ALLOC(ws.d_flags, 8);
  ws.orphan_cap = 1 << 16;
  WS_ALLOC(ws.orphans, ws.orphan_cap);
  // the split count depends on N: size for both the request and the headroom
  const size_t sc = std::max(scratch, gpr_scratch_bytes(nN, m->host.M, D, sizeof(double)));
  if (sc > 0) {
    if (cudaMalloc(&ws.gpr_scratch, sc) != cudaSuccess) {
      free_ws(ws);
      return fail(GAPGB_ERR_ALLOC, "cudaMalloc failed for GPR scratch");
    }
  }
  ws.gpr_scratch_size = sc;
  ws.tc_scratch_size = std::max(tc_atom_scratch_bytes(nN), tf32_atom_scratch_bytes(nN));
  if (cudaMalloc(&ws.tc_scratch, ws.tc_scratch_size) != cudaSuccess) {
    free_ws(ws);
    return fail(GAPGB_ERR_ALLOC, "cudaMalloc failed for tensor-core scratch");
  }
  if (cudaMallocHost((void **)&ws.h_flags, 8 * sizeof(int)) != cudaSuccess) {
    free_ws(ws);
    return fail(GAPGB_ERR_ALLOC, "cudaMallocHost failed");
  }
  ws.N = nN;
  ws.S = nS;
  ws.cap = nC;
  ws.D = D;
  return GAPGB_OK;
}

// Host-side validation at model creation (no device work).
gapgb_status validate_model(gapgb_model *m) {
  const HostModel &h = m->host;
  std::string err;
  gapgb_status st = build_sf_table(h, &m->sfh, &err);
  if (st) return fail(st, err);
  if (h.D > 128) return fail(GAPGB_ERR_CAP_EXCEEDED, "descriptor length D > 128");
  for (int d = 0; d < h.D; ++d)
    if (!(h.theta[d] != 0.0) || !std::isfinite(h.theta[d]))
      return fail(GAPGB_ERR_PARSE, "theta must be finite and non-zero");
  return GAPGB_OK;
}

// Device upload, done by the first call that needs the GPU.
gapgb_status upload_model(gapgb_model *m) {
  if (m->d_sf) return GAPGB_OK;
  const HostModel &h = m->host;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
    return fail(GAPGB_ERR_NO_DEVICE, "no CUDA device visible");
  if (m->device < 0 || m->device >= ndev) return fail(GAPGB_ERR_ARG, "device ordinal out of range");
  GAPGB_CUDA_TRY(cudaSetDevice(m->device));
  const int M = h.M, D = h.D;
  std::vector<double> mmt((size_t)M * D), invth(D);
  std::vector<float> mmt32((size_t)M * D), invth32(D), coeff32(M);
  for (int d = 0; d < D; ++d) {
    invth[d] = 1.0 / h.theta[d];
    invth32[d] = (float)invth[d];
  }
  for (int k = 0; k < M; ++k) {
    coeff32[k] = (float)h.coeff[k];
    for (int d = 0; d < D; ++d) {
      mmt[(size_t)k * D + d] = h.mm[(size_t)k * D + d] / h.theta[d];
      mmt32[(size_t)k * D + d] = (float)mmt[(size_t)k * D + d];
    }
  }
  SFDev *d_sf = nullptr;
  GAPGB_CUDA_TRY(cudaMalloc(&d_sf, sizeof(SFDev)));
  GAPGB_CUDA_TRY(cudaMemcpy(d_sf, &m->sfh, sizeof(SFDev), cudaMemcpyHostToDevice));
  const SFT<double> t64 = make_sft<double>(m->sfh);
  const SFT<float> t32 = make_sft<float>(m->sfh);
  m->sft32h = t32;
  GAPGB_CUDA_TRY(cudaMalloc(&m->d_sft64, sizeof(t64)));
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_sft64, &t64, sizeof(t64), cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMalloc(&m->d_sft32, sizeof(t32)));
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_sft32, &t32, sizeof(t32), cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMalloc(&m->d_mmt, sizeof(double) * mmt.size()));
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_mmt, mmt.data(), sizeof(double) * mmt.size(), cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMalloc(&m->d_mmt32, sizeof(float) * mmt32.size()));
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_mmt32, mmt32.data(), sizeof(float) * mmt32.size(), cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMalloc(&m->d_invth, sizeof(double) * D));
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_invth, invth.data(), sizeof(double) * D, cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMalloc(&m->d_invth32, sizeof(float) * D));
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_invth32, invth32.data(), sizeof(float) * D, cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMalloc(&m->d_coeff, sizeof(double) * M));
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_coeff, h.coeff.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMalloc(&m->d_coeff32, sizeof(float) * M));
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_coeff32, coeff32.data(), sizeof(float) * M, cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  for (auto &e : m->ev) GAPGB_CUDA_TRY(cudaEventCreate(&e));
  GAPGB_CUDA_TRY(cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking));
  GAPGB_CUDA_TRY(cudaEventCreateWithFlags(&m->ev_fork, cudaEventDisableTiming));
  GAPGB_CUDA_TRY(cudaEventCreateWithFlags(&m->ev_join, cudaEventDisableTiming));
  const char *prof = std::getenv("GAPGB_PROFILE_STAGES");
  m->profile_stages = prof && prof[0] && prof[0] != '0';
  m->d_sf = d_sf;  // marks the model as uploaded
  return GAPGB_OK;
}

int max_struct_atoms(int S, const int *atom_off) {
  int mx = 0;
  for (int s = 0; s < S; ++s) mx = std::max(mx, atom_off[s + 1] - atom_off[s]);
  return mx;
}

// A double is not finite exactly when its exponent field (bits 20..30 of the
// high 32-bit word) is all ones.  The largest masked high word of a block is
// an unsigned-max reduction the host compiler vectorises (one pass over the
// positions of the call, on its critical path before the first launch).
bool finite_all(const double *p, size_t n) {
  constexpr uint32_t kExp = 0x7FF00000u;
  constexpr size_t kBlock = 4096;
  for (size_t b = 0; b < n; b += kBlock) {
    const size_t e = std::min(n, b + kBlock);
    uint32_t mx = 0;
    for (size_t i = b; i < e; ++i) {
      uint64_t u;
      std::memcpy(&u, p + i, sizeof(u));
      const uint32_t x = static_cast<uint32_t>(u >> 32) & kExp;
      mx = x > mx ? x : mx;
    }
    if (mx == kExp) return false;
  }
  return true;
}

// the batch's structure offsets (cheap: one pass over nstruct entries)
gapgb_status check_offsets_host(int nstruct, const int *atom_off) {
  if (nstruct <= 0 || !atom_off) return fail(GAPGB_ERR_ARG, "nstruct must be positive");
  if (atom_off[0] != 0) return fail(GAPGB_ERR_ARG, "atom_off[0] must be 0");
  for (int s = 0; s < nstruct; ++s)
    if (atom_off[s + 1] <= atom_off[s]) return fail(GAPGB_ERR_ARG, "every structure needs at least one atom");
  return GAPGB_OK;
}

// finite lattices and positions, non-singular lattices (one pass over the
// positions: the host path runs it while the inputs are being copied)
gapgb_status check_geometry_host(int nstruct, const int *atom_off, const double *lat,
                                 const double *pos) {
  if (!finite_all(lat, (size_t)nstruct * 9)) return fail(GAPGB_ERR_ARG, "non-finite lattice");
  if (!finite_all(pos, (size_t)atom_off[nstruct] * 3)) return fail(GAPGB_ERR_ARG, "non-finite position");
  for (int s = 0; s < nstruct; ++s) {
    const double *L = lat + (size_t)s * 9;
    const double det = L[0] * (L[4] * L[8] - L[5] * L[7]) - L[1] * (L[3] * L[8] - L[5] * L[6]) +
                       L[2] * (L[3] * L[7] - L[4] * L[6]);
    if (!(std::fabs(det) > 0.0)) return fail(GAPGB_ERR_ARG, "singular lattice");
  }
  return GAPGB_OK;
}

gapgb_status check_batch_host(int nstruct, const int *atom_off, const double *lat,
                              const double *pos) {
  gapgb_status st = check_offsets_host(nstruct, atom_off);
  return st ? st : check_geometry_host(nstruct, atom_off, lat, pos);
}

// Everything after the neighbour list, enqueued on `st`.
// Fallback buffers of the surrogate form for N atoms (allocates; runs before
// any capture, so a captured evaluation finds them sized).
gapgb_status ensure_surrogate(gapgb_model *m, int N) {
  if (!m->surrogate) return fail(GAPGB_ERR_ARG, "no surrogate attached to the model");
  gapgb_status st = surrogate_prepare(m->surrogate, N);
  if (st) return st;
  if (N <= m->surr_cap) return GAPGB_OK;
  if (m->live_graphs->load() > 0)
    return fail(GAPGB_ERR_ARG, "surrogate buffers would move while a CUDA graph is alive");
  free_dev(m->surr_std);
  free_dev(m->surr_gstd);
  free_dev(m->fb_rows);
  free_dev(m->fb_count);
  free_dev(m->fb_scratch);
  m->surr_cap = 0;
  const int n = N + N / 8;
  if (cudaMalloc(&m->surr_std, sizeof(float) * n) != cudaSuccess ||
      cudaMalloc(&m->surr_gstd, sizeof(float) * n) != cudaSuccess ||
      cudaMalloc(&m->fb_rows, sizeof(int) * n) != cudaSuccess ||
      cudaMalloc(&m->fb_count, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&m->fb_scratch, gpr_rows_scratch_bytes(n, m->host.D)) != cudaSuccess) {
    cudaGetLastError();
    return fail(GAPGB_ERR_ALLOC, "cudaMalloc failed for the surrogate fallback buffers");
  }
  m->surr_cap = n;
  return GAPGB_OK;
}

// Two pipelines: atoms [0, h) on `st` and [h, N) on the model's side stream
// (h a multiple of the 128-atom GPR tile), each running descriptors -> GPR ->
// slot gradients, joined before the structure sums.  The halves touch
// disjoint per-atom ranges of the workspace; the force scatter of both adds
// into the one force array (FP64 atomics), zeroed before the fork.  The
// fork / join are event waits, so the pair of streams is captured into a
// CUDA graph like a single stream.
constexpr int kSplitMinAtoms = 20480;

bool split_applies(const gapgb_model *m, int N, int lgrad) {
  return m->pipelines == 2 && !m->profile_stages && lgrad && N >= kSplitMinAtoms &&
         (m->precision == GAPGB_PREC_TC || m->precision == GAPGB_PREC_TF32) &&
         bwd_scatters_forces(m);
}

gapgb_status enqueue_split(gapgb_model *m, int S, int N, int cap, int capS,
                           double *d_energy, double *d_force, double *d_stress,
                           double *d_atom_e, cudaStream_t st) {
  Workspace &ws = m->ws;
  const bool tc = m->precision == GAPGB_PREC_TC;
  gapgb_status s = tc ? build_tc_image(m) : build_tf32_image(m);  // first call only (allocates)
  if (s) return s;
  const int h = (N / 2) / 128 * 128;
  cudaMemsetAsync(d_force, 0, sizeof(double) * 3 * (size_t)N, st);
  cudaEventRecord(m->ev_fork, st);
  cudaStreamWaitEvent(m->side, m->ev_fork, 0);
  const int lo[2] = {0, h}, hi[2] = {h, N};
  cudaStream_t ss[2] = {st, m->side};
  for (int p = 0; p < 2; ++p) {
    launch_wacsf_fwd<float>(m, ws, N, cap, capS, ss[p], lo[p], hi[p]);
    if (tc) launch_gpr_tc(m, ws, N, ss[p], lo[p], hi[p]);
    else launch_gpr_tf32(m, ws, N, ss[p], lo[p], hi[p]);
    launch_wacsf_bwd<float>(m, ws, N, cap, capS, d_force, ss[p], lo[p], hi[p], false);
  }
  cudaEventRecord(m->ev_join, m->side);
  cudaStreamWaitEvent(st, m->ev_join, 0);
  launch_struct_reduce(ws, S, 1, d_energy, d_stress, d_atom_e, N, st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GAPGB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return GAPGB_OK;
}

gapgb_status enqueue_tail(gapgb_model *m, int S, int N, int cap, int capS, int lgrad,
                          const int *d_species, double *d_energy, double *d_force,
                          double *d_stress, double *d_atom_e, cudaStream_t st) {
  if (split_applies(m, N, lgrad))
    return enqueue_split(m, S, N, cap, capS, d_energy, d_force, d_stress, d_atom_e, st);
  Workspace &ws = m->ws;
  const bool prof = m->profile_stages;
  // reverse slots serve the force gather only
  if (lgrad && !bwd_scatters_forces(m)) launch_reverse(ws, N, cap, st);
  if (prof) cudaEventRecord(m->ev[1], st);
  const bool fp64 = m->precision == GAPGB_PREC_FP64;
  if (fp64) launch_wacsf_fwd<double>(m, ws, N, cap, capS, st);
  else launch_wacsf_fwd<float>(m, ws, N, cap, capS, st);
  if (prof) cudaEventRecord(m->ev[2], st);
  if (m->precision == GAPGB_PREC_SURROGATE) {
    // committee for every atom, then the exact GPR for the atoms it flags
    surrogate_enqueue(m->surrogate, N, d_species, (const float *)ws.G, ws.e, m->surr_std,
                      (float *)ws.dedg, m->surr_gstd, ws.d_flags, st);
    surrogate_select_fallback(N, m->surr_std, (float)m->surr_threshold, m->surr_gstd,
                              (float)m->surr_gspread, ws.nbr_cnt, ws.nbr_d32, cap,
                              (float)m->surr_contact, m->fb_rows, m->fb_count, st);
    launch_gpr_rows(m, ws, m->surr_cap, m->fb_rows, m->fb_count, m->fb_scratch, st);
  }
  else if (m->precision == GAPGB_PREC_TC) {
    gapgb_status s = build_tc_image(m);  // first call only (allocates)
    if (s) return s;
    launch_gpr_tc(m, ws, N, st);
  }
  else if (m->precision == GAPGB_PREC_TF32) {
    gapgb_status s = build_tf32_image(m);  // first call only (allocates)
    if (s) return s;
    launch_gpr_tf32(m, ws, N, st);
  }
  else if (fp64) launch_gpr<double, double>(m, ws, N, st);
  else if (m->precision == GAPGB_PREC_MIXED) launch_gpr<double, float>(m, ws, N, st);
  else launch_gpr<float, float>(m, ws, N, st);
  if (prof) cudaEventRecord(m->ev[3], st);
  if (lgrad) {
    if (fp64) {
      launch_wacsf_bwd<double>(m, ws, N, cap, capS, d_force, st);
      launch_forces<double>(ws, N, cap, d_force, st);
    } else {
      if (!launch_wacsf_bwd<float>(m, ws, N, cap, capS, d_force, st))
        launch_forces<float>(ws, N, cap, d_force, st);
    }
  } else {
    cudaMemsetAsync(d_force, 0, sizeof(double) * 3 * (size_t)N, st);
  }
  launch_struct_reduce(ws, S, lgrad, d_energy, d_stress, d_atom_e, N, st);
  if (prof) cudaEventRecord(m->ev[4], st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GAPGB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return GAPGB_OK;
}

__global__ void k_d2f(size_t n, const double *__restrict__ a, float *__restrict__ b) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

gapgb_status flags_to_status(const int *f) {
  if (f[0] & kFlagUnknownSpecies) return fail(GAPGB_ERR_UNKNOWN_SPECIES, "atomic number not in the model's species table");
  if (f[0] & kFlagImageLimit) return fail(GAPGB_ERR_CAP_EXCEEDED, "more than 127 periodic images per lattice direction");
  if (f[0] & kFlagNeighbourOverflow) return fail(GAPGB_ERR_NEIGHBOUR_OVERFLOW, "neighbour capacity exceeded (max count " + std::to_string(f[1]) + ")");
  if (f[0] & kFlagOrphanOverflow) return fail(GAPGB_ERR_CAP_EXCEEDED, "too many unpaired neighbour slots");
  if (f[0] & kFlagTimeout) return fail(GAPGB_ERR_TIMEOUT, "a bounded device wait gave up");
  if (f[0] & kFlagNotPositiveDefinite)
    return fail(GAPGB_ERR_ARG, "the fit's normal matrix is not positive definite (raise the jitter)");
  if (f[0] & kFlagForceRange)
    return fail(GAPGB_ERR_CAP_EXCEEDED,
                "a slot-gradient term beyond 2047 eV/A or not finite (FP32 forms); use the FP64 form");
  if (f[0] & kFlagSkinExceeded)
    return fail(GAPGB_ERR_CAP_EXCEEDED, "an atom moved more than half the Verlet skin between rebuilds");
  return GAPGB_OK;
}

void read_stage_times(gapgb_model *m) {
  if (!m->profile_stages) return;
  cudaEventSynchronize(m->ev[4]);
  for (int q = 0; q < 4; ++q) cudaEventElapsedTime(&m->stage_ms[q], m->ev[q], m->ev[q + 1]);
}

// Host-buffer path: copies, neighbour list, one sync, the rest, copies back.
gapgb_status eval_host(gapgb_model *m, int S, const int *atom_off, const int *species,
                       const double *lat, const double *pos, int lgrad, double *energy,
                       double *force, double *stress, double *atom_e, double **d_G_out) {
  gapgb_status st = check_offsets_host(S, atom_off);
  if (st) return st;
  if (!lat || !pos) return fail(GAPGB_ERR_ARG, "null argument");
  const int N = atom_off[S];
  st = upload_model(m);
  if (st) return st;
  GAPGB_CUDA_TRY(cudaSetDevice(m->device));
  st = ensure_ws(m, N, S, m->cap);
  if (st) return st;
  Workspace &ws = m->ws;
  cudaStream_t s = m->stream;
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_atom_off, atom_off, sizeof(int) * (S + 1), cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_species, species, sizeof(int) * N, cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_lat, lat, sizeof(double) * 9 * S, cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_pos, pos, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s));
  // the geometry checks run on the host while the copies are in flight; no
  // kernel is launched before they pass
  st = check_geometry_host(S, atom_off, lat, pos);
  if (st) {
    cudaStreamSynchronize(s);  // the copies read the caller's buffers
    return st;
  }
  const int maxa = max_struct_atoms(S, atom_off);
  // the slot count the descriptor kernels are sized for: the previous call's
  // maximum, or on a model's first call the whole capacity (a bound on any
  // count that does not overflow it), so the first call also synchronises once
  const int caps_guess = m->caps_hint > 0 ? m->caps_hint : (m->cap <= 256 ? m->cap : 0);
  if (!d_G_out && caps_guess > 0 && caps_guess <= m->cap) {
    // one synchronisation: the descriptor kernels take that slot count; the
    // neighbour kernel reports the true maximum, and a batch that needs more
    // slots (or overflows the capacity) is recomputed by the general path below
    const int cap = m->cap, capS = caps_guess;
    if (m->precision == GAPGB_PREC_SURROGATE) {
      st = ensure_surrogate(m, N);
      if (st) return st;
    }
    GAPGB_CUDA_TRY(cudaMemsetAsync(ws.d_flags, 0, 8 * sizeof(int), s));
    if (m->profile_stages) cudaEventRecord(m->ev[0], s);
    launch_prep(m, ws, S, N, ws.d_atom_off, ws.d_species, ws.d_lat, ws.d_pos, m->host.rcut, s,
                maxa >= kBinMinAtoms);
    launch_neighbors(ws, S, N, maxa, cap, m->host.rcut, s, m->precision == GAPGB_PREC_FP64);
    st = enqueue_tail(m, S, N, cap, capS, lgrad, ws.d_species, ws.d_energy, ws.d_force,
                      ws.d_stress, ws.d_atom_e, s);
    if (st) return st;
    GAPGB_CUDA_TRY(cudaMemcpyAsync(energy, ws.d_energy, sizeof(double) * S, cudaMemcpyDeviceToHost, s));
    if (force) GAPGB_CUDA_TRY(cudaMemcpyAsync(force, ws.d_force, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s));
    if (stress) GAPGB_CUDA_TRY(cudaMemcpyAsync(stress, ws.d_stress, sizeof(double) * 6 * S, cudaMemcpyDeviceToHost, s));
    if (atom_e) GAPGB_CUDA_TRY(cudaMemcpyAsync(atom_e, ws.d_atom_e, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.h_flags, ws.d_flags, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
    GAPGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (!(ws.h_flags[0] & kFlagNeighbourOverflow) && ws.h_flags[1] <= capS) {
      read_stage_times(m);
      m->caps_hint = std::min(cap, std::max(8, (ws.h_flags[1] + 7) / 8 * 8));
      return flags_to_status(ws.h_flags);
    }
  }
  for (int attempt = 0; attempt < 3; ++attempt) {
    const int cap = m->cap;
    GAPGB_CUDA_TRY(cudaMemsetAsync(ws.d_flags, 0, 8 * sizeof(int), s));
    if (m->profile_stages) cudaEventRecord(m->ev[0], s);
    launch_prep(m, ws, S, N, ws.d_atom_off, ws.d_species, ws.d_lat, ws.d_pos, m->host.rcut, s,
                maxa >= kBinMinAtoms);
    launch_neighbors(ws, S, N, maxa, cap, m->host.rcut, s,
                     m->precision == GAPGB_PREC_FP64 || d_G_out != nullptr);
    GAPGB_CUDA_TRY(cudaGetLastError());
    GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.h_flags, ws.d_flags, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
    GAPGB_CUDA_TRY(cudaStreamSynchronize(s));
    const int maxcnt = ws.h_flags[1];
    // unknown species and the image limit end the call before any growth (a
    // clamped image range can overflow every capacity)
    if (ws.h_flags[0] & (kFlagUnknownSpecies | kFlagImageLimit)) return flags_to_status(ws.h_flags);
    if (ws.h_flags[0] & kFlagNeighbourOverflow) {
      const int newcap = ((maxcnt + 31) / 32) * 32;
      m->cap = newcap;
      st = ensure_ws(m, N, S, newcap);
      if (st) return st;
      continue;
    }
    st = flags_to_status(ws.h_flags);
    if (st) return st;
    const int capS = maxcnt > 0 ? maxcnt : 1;
    if (d_G_out) {
      // descriptors only (gapgb_descriptors, gapgb_variance, gapgb_fit_energies)
      if (m->precision == GAPGB_PREC_FP64) launch_wacsf_fwd<double>(m, ws, N, cap, capS, s);
      else launch_wacsf_fwd<float>(m, ws, N, cap, capS, s);
      GAPGB_CUDA_TRY(cudaGetLastError());
      *d_G_out = (double *)ws.G;
      GAPGB_CUDA_TRY(cudaStreamSynchronize(s));
      return GAPGB_OK;
    }
    if (m->precision == GAPGB_PREC_SURROGATE) {
      st = ensure_surrogate(m, N);
      if (st) return st;
    }
    st = enqueue_tail(m, S, N, cap, capS, lgrad, ws.d_species, ws.d_energy, ws.d_force,
                      ws.d_stress, ws.d_atom_e, s);
    if (st) return st;
    GAPGB_CUDA_TRY(cudaMemcpyAsync(energy, ws.d_energy, sizeof(double) * S, cudaMemcpyDeviceToHost, s));
    if (force) GAPGB_CUDA_TRY(cudaMemcpyAsync(force, ws.d_force, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s));
    if (stress) GAPGB_CUDA_TRY(cudaMemcpyAsync(stress, ws.d_stress, sizeof(double) * 6 * S, cudaMemcpyDeviceToHost, s));
    if (atom_e) GAPGB_CUDA_TRY(cudaMemcpyAsync(atom_e, ws.d_atom_e, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.h_flags, ws.d_flags, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
    GAPGB_CUDA_TRY(cudaStreamSynchronize(s));
    read_stage_times(m);
    m->caps_hint = std::min(cap, std::max(8, (maxcnt + 7) / 8 * 8));
    return flags_to_status(ws.h_flags);
  }
  return fail(GAPGB_ERR_NEIGHBOUR_OVERFLOW, "neighbour capacity could not be grown");
}

}  // namespace

// ---- molecular dynamics support (md.cu) ------------------------------------

gapgb_status md_prepare(gapgb_model *m, int N, int S) {
  gapgb_status st = upload_model(m);
  if (st) return st;
  GAPGB_CUDA_TRY(cudaSetDevice(m->device));
  st = ensure_ws(m, N, S, m->cap);
  if (st) return st;
  if (m->precision == GAPGB_PREC_SURROGATE) return ensure_surrogate(m, N);
  return GAPGB_OK;
}

// One evaluation of an MD step: the neighbour list is built with cutoff
// rcut + skin (rebuild) or refreshed from the current positions (otherwise).
// Error bits accumulate in flags[0] across steps; the per-pass counters are
// reset here.  Never synchronises or allocates (md_prepare sized everything).
gapgb_status md_eval_enqueue(gapgb_model *m, int S, int N, const int *d_atom_off,
                             const int *d_species, const double *d_lat, const double *d_pos,
                             bool rebuild, double skin, double *d_energy, double *d_force,
                             double *d_stress, cudaStream_t s) {
  Workspace &ws = m->ws;
  const double rb = m->host.rcut + skin;
  GAPGB_CUDA_TRY(cudaMemsetAsync(ws.d_flags + 1, 0, 2 * sizeof(int), s));
  launch_prep(m, ws, S, N, d_atom_off, d_species, d_lat, d_pos, rb, s, rebuild && N >= kBinMinAtoms);
  if (rebuild) launch_neighbors(ws, S, N, N, m->cap, rb, s, m->precision == GAPGB_PREC_FP64);
  else launch_refresh(ws, N, m->cap, s, m->precision == GAPGB_PREC_FP64);
  return enqueue_tail(m, S, N, m->cap, m->cap, 1, d_species, d_energy, d_force, d_stress, nullptr,
                      s);
}

gapgb_status md_read_flags(gapgb_model *m, int *max_count) {
  Workspace &ws = m->ws;
  GAPGB_CUDA_TRY(cudaMemcpy(ws.h_flags, ws.d_flags, 8 * sizeof(int), cudaMemcpyDeviceToHost));
  if (max_count) *max_count = ws.h_flags[1];
  return flags_to_status(ws.h_flags);
}

gapgb_status md_clear_flags(gapgb_model *m) {
  GAPGB_CUDA_TRY(cudaMemset(m->ws.d_flags, 0, 8 * sizeof(int)));
  return GAPGB_OK;
}

}  // namespace gapgb

using namespace gapgb;

extern "C" {

const char *gapgb_status_string(gapgb_status st) {
  switch (st) {
    case GAPGB_OK: return "ok";
    case GAPGB_ERR_FILE: return "model file missing or unreadable";
    case GAPGB_ERR_PARSE: return "model file malformed";
    case GAPGB_ERR_CAP_EXCEEDED: return "size beyond a documented limit";
    case GAPGB_ERR_UNKNOWN_SPECIES: return "atomic number absent from the model";
    case GAPGB_ERR_NEIGHBOUR_OVERFLOW: return "neighbour capacity exceeded";
    case GAPGB_ERR_CUDA: return "CUDA error";
    case GAPGB_ERR_TIMEOUT: return "device wait timed out";
    case GAPGB_ERR_ARG: return "invalid argument";
    case GAPGB_ERR_ALLOC: return "allocation failed";
    case GAPGB_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

const char *gapgb_last_error(void) { return g_last_error.c_str(); }

const char *gapgb_version(void) { return "gapgb 0.1 (sm_103a)"; }

gapgb_status gapgb_model_load(const char *path, double rcut, gapgb_model **out) {
  if (!path || !out) return fail(GAPGB_ERR_ARG, "null argument");
  *out = nullptr;
  if (!(rcut > 0.0)) return fail(GAPGB_ERR_ARG, "rcut must be positive");
  gapgb_model *m = new gapgb_model();
  std::string err;
  gapgb_status st = parse_model_file(path, &m->host, &err);
  if (st) {
    delete m;
    return fail(st, err);
  }
  m->host.rcut = rcut;
  st = validate_model(m);
  if (st) {
    gapgb_model_free(m);
    return st;
  }
  *out = m;
  return GAPGB_OK;
}

gapgb_status gapgb_model_write(const gapgb_model *model, const char *path) {
  if (!model || !path) return fail(GAPGB_ERR_ARG, "null argument");
  std::string err;
  const gapgb_status st = write_model_file(model->host, path, &err);
  return st ? fail(st, err) : GAPGB_OK;
}

gapgb_status gapgb_model_create(int nspecies, const int *species_z, const double *species_w,
                                int nsf, const int *sf_type, const double *sf_alpha,
                                const double *sf_cutoff, const double *sf_zeta, int nsparse,
                                int des_len, const double *theta, const double *mm,
                                const double *coeff, double rcut, gapgb_model **out) {
  if (!out || !species_z || !species_w || !sf_type || !sf_alpha || !sf_cutoff || !theta || !mm ||
      !coeff)
    return fail(GAPGB_ERR_ARG, "null argument");
  *out = nullptr;
  if (nspecies <= 0 || nsf <= 0 || nsf > kMaxSF || nsparse <= 0 || des_len <= 0 || !(rcut > 0.0))
    return fail(GAPGB_ERR_ARG, "sizes must be positive (nsf <= 128)");
  gapgb_model *m = new gapgb_model();
  HostModel &h = m->host;
  h.nspecies = nspecies;
  h.species_z.assign(species_z, species_z + nspecies);
  h.species_w.assign(species_w, species_w + nspecies);
  h.nsf = nsf;
  h.sf_type.assign(sf_type, sf_type + nsf);
  h.sf_alpha.assign(sf_alpha, sf_alpha + nsf);
  h.sf_cutoff.assign(sf_cutoff, sf_cutoff + nsf);
  h.sf_zeta.assign(nsf, 1.0);
  if (sf_zeta) h.sf_zeta.assign(sf_zeta, sf_zeta + nsf);
  h.M = nsparse;
  h.D = des_len;
  h.theta.assign(theta, theta + des_len);
  h.mm.assign(mm, mm + (size_t)nsparse * des_len);
  h.coeff.assign(coeff, coeff + nsparse);
  h.rcut = rcut;
  gapgb_status st = validate_model(m);
  if (st) {
    gapgb_model_free(m);
    return st;
  }
  *out = m;
  return GAPGB_OK;
}

void gapgb_model_free(gapgb_model *m) {
  if (!m) return;
  cudaSetDevice(m->device);
  free_ws(m->ws);
  free_dev(m->d_sf);
  free_dev(m->d_sft64);
  free_dev(m->d_sft32);
  free_dev(m->d_mmt);
  free_dev(m->d_mmt32);
  free_dev(m->d_invth);
  free_dev(m->d_invth32);
  free_dev(m->d_coeff);
  free_dev(m->d_coeff32);
  free_dev(m->surr_std);
  free_dev(m->surr_gstd);
  free_dev(m->fb_rows);
  free_dev(m->fb_count);
  free_dev(m->fb_scratch);
  if (m->d_tc) cudaFree(m->d_tc);
  if (m->d_tf32) cudaFree(m->d_tf32);
  variance_free(m->var);
  for (auto &e : m->ev)
    if (e) cudaEventDestroy(e);
  if (m->ev_fork) cudaEventDestroy(m->ev_fork);
  if (m->ev_join) cudaEventDestroy(m->ev_join);
  if (m->stream) cudaStreamDestroy(m->stream);
  if (m->side) cudaStreamDestroy(m->side);
  delete m;
}

gapgb_status gapgb_model_info(const gapgb_model *m, int *nsparse, int *des_len, int *nsf,
                              int *nspecies, double *rcut) {
  if (!m) return fail(GAPGB_ERR_ARG, "null model");
  if (nsparse) *nsparse = m->host.M;
  if (des_len) *des_len = m->host.D;
  if (nsf) *nsf = m->host.nsf;
  if (nspecies) *nspecies = m->host.nspecies;
  if (rcut) *rcut = m->host.rcut;
  return GAPGB_OK;
}

gapgb_status gapgb_model_arrays(const gapgb_model *m, double *theta, double *mm, double *coeff) {
  if (!m) return fail(GAPGB_ERR_ARG, "null model");
  if (theta) std::memcpy(theta, m->host.theta.data(), sizeof(double) * m->host.D);
  if (mm) std::memcpy(mm, m->host.mm.data(), sizeof(double) * m->host.mm.size());
  if (coeff) std::memcpy(coeff, m->host.coeff.data(), sizeof(double) * m->host.M);
  return GAPGB_OK;
}

gapgb_status gapgb_model_tables(const gapgb_model *m, int *species_z, double *species_w,
                                int *sf_type, double *sf_alpha, double *sf_cutoff,
                                double *sf_zeta) {
  if (!m) return fail(GAPGB_ERR_ARG, "null model");
  const HostModel &h = m->host;
  if (species_z) std::memcpy(species_z, h.species_z.data(), sizeof(int) * h.nspecies);
  if (species_w) std::memcpy(species_w, h.species_w.data(), sizeof(double) * h.nspecies);
  if (sf_type) std::memcpy(sf_type, h.sf_type.data(), sizeof(int) * h.nsf);
  if (sf_alpha) std::memcpy(sf_alpha, h.sf_alpha.data(), sizeof(double) * h.nsf);
  if (sf_cutoff) std::memcpy(sf_cutoff, h.sf_cutoff.data(), sizeof(double) * h.nsf);
  if (sf_zeta) std::memcpy(sf_zeta, h.sf_zeta.data(), sizeof(double) * h.nsf);
  return GAPGB_OK;
}

gapgb_status gapgb_set_option(gapgb_model *m, gapgb_option opt, int64_t value) {
  if (!m) return fail(GAPGB_ERR_ARG, "null model");
  if (m->live_graphs->load() > 0 && opt != GAPGB_OPT_DEVICE)
    return fail(GAPGB_ERR_ARG, "the model is bound to a live CUDA graph (free it first)");
  switch (opt) {
    case GAPGB_OPT_PRECISION:
      if (value != GAPGB_PREC_FP64 && value != GAPGB_PREC_FP32 && value != GAPGB_PREC_MIXED &&
          value != GAPGB_PREC_TC && value != GAPGB_PREC_SURROGATE && value != GAPGB_PREC_TF32)
        return fail(GAPGB_ERR_ARG, "unknown precision");
      if (value == GAPGB_PREC_TF32 && m->host.D > 64)
        return fail(GAPGB_ERR_CAP_EXCEEDED, "tensor-core GPR supports D <= 64");
      if (value == GAPGB_PREC_SURROGATE && !m->surrogate)
        return fail(GAPGB_ERR_ARG, "attach a surrogate (gapgb_model_set_surrogate) first");
      if (value == GAPGB_PREC_TC && m->host.D > 64)
        return fail(GAPGB_ERR_CAP_EXCEEDED, "tensor-core GPR supports D <= 64");
      m->precision = (int)value;
      return GAPGB_OK;
    case GAPGB_OPT_NEIGHBOUR_CAP:
      if (value < 1 || value > 65536) return fail(GAPGB_ERR_ARG, "capacity out of range");
      m->cap = (int)value;
      return GAPGB_OK;
    case GAPGB_OPT_DEVICE:
      return fail(GAPGB_ERR_ARG, "the device is fixed when the model is created");
    case GAPGB_OPT_GENERIC_KERNELS:
      m->generic_kernels = value != 0;
      return GAPGB_OK;
    case GAPGB_OPT_PIPELINES:
      if (value != 1 && value != 2) return fail(GAPGB_ERR_ARG, "pipelines must be 1 or 2");
      m->pipelines = (int)value;
      return GAPGB_OK;
  }
  return fail(GAPGB_ERR_ARG, "unknown option");
}

gapgb_status gapgb_get_option(const gapgb_model *m, gapgb_option opt, int64_t *value) {
  if (!m || !value) return fail(GAPGB_ERR_ARG, "null argument");
  switch (opt) {
    case GAPGB_OPT_PRECISION: *value = m->precision; return GAPGB_OK;
    case GAPGB_OPT_NEIGHBOUR_CAP: *value = m->cap; return GAPGB_OK;
    case GAPGB_OPT_DEVICE: *value = m->device; return GAPGB_OK;
    case GAPGB_OPT_GENERIC_KERNELS: *value = m->generic_kernels ? 1 : 0; return GAPGB_OK;
    case GAPGB_OPT_PIPELINES: *value = m->pipelines; return GAPGB_OK;
  }
  return fail(GAPGB_ERR_ARG, "unknown option");
}

gapgb_status gapgb_eval(gapgb_model *m, int natoms, const int *species, const double *lat,
                        const double *pos, int lgrad, double *energy, double *force,
                        double *stress, double *variance) {
  if (!m || !species || !lat || !pos || !energy) return fail(GAPGB_ERR_ARG, "null argument");
  if (natoms <= 0) return fail(GAPGB_ERR_ARG, "natoms must be positive");
  if (lgrad && (!force || !stress)) return fail(GAPGB_ERR_ARG, "force and stress needed with lgrad");
  const int off[2] = {0, natoms};
  double stress_local[6];
  gapgb_status st = eval_host(m, 1, off, species, lat, pos, lgrad, energy, force,
                              stress ? stress : stress_local, nullptr, nullptr);
  if (variance) *variance = 0.0;  // gap_calc.f90:206
  if (st || !variance || m->var.qmm.empty()) return st;
  // a qmm is attached: the variance block of gap_calc.f90:207-210 on this
  // evaluation's descriptors
  cudaStream_t s = m->stream;
  st = variance_enqueue(m, 1, natoms, m->ws.d_atom_off, m->ws.G,
                        m->precision == GAPGB_PREC_FP64, s);
  if (st) return st;
  GAPGB_CUDA_TRY(cudaMemcpyAsync(variance, m->var.var, sizeof(double), cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(m->ws.h_flags, m->ws.d_flags, 8 * sizeof(int),
                                 cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaStreamSynchronize(s));
  return flags_to_status(m->ws.h_flags);
}

gapgb_status gapgb_model_set_coeff(gapgb_model *m, const double *coeff) {
  if (!m || !coeff) return fail(GAPGB_ERR_ARG, "null argument");
  const int M = m->host.M;
  for (int k = 0; k < M; ++k)
    if (!std::isfinite(coeff[k])) return fail(GAPGB_ERR_ARG, "coefficients must be finite");
  m->host.coeff.assign(coeff, coeff + M);
  if (!m->d_sf) return GAPGB_OK;  // not on the device yet: the upload takes the new values
  GAPGB_CUDA_TRY(cudaSetDevice(m->device));
  GAPGB_CUDA_TRY(cudaStreamSynchronize(m->stream));
  std::vector<float> c32(M);
  for (int k = 0; k < M; ++k) c32[k] = (float)coeff[k];
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_coeff, coeff, sizeof(double) * M, cudaMemcpyHostToDevice));
  GAPGB_CUDA_TRY(cudaMemcpy(m->d_coeff32, c32.data(), sizeof(float) * M, cudaMemcpyHostToDevice));
  // the tensor-core operand images carry c: rewritten in place, so graphs
  // that captured them replay with the new coefficients
  if (m->d_tc) {
    const gapgb_status st = build_tc_image(m, true);
    if (st) return st;
  }
  if (m->d_tf32) {
    const gapgb_status st = build_tf32_image(m, true);
    if (st) return st;
  }
  return GAPGB_OK;
}

gapgb_status gapgb_fit(gapgb_model *m, int nstruct, const int *atom_off, const int *species,
                       const double *lat, const double *pos, const double *energy,
                       const double *forces, const double *stress, double sigma_e,
                       double sigma_f, double sigma_s, double jitter, double *coeff) {
  if (!m || !atom_off || !species || !lat || !pos || !energy)
    return fail(GAPGB_ERR_ARG, "null argument");
  if (!(sigma_e > 0.0) || !(jitter >= 0.0) || (forces && !(sigma_f > 0.0)) ||
      (stress && !(sigma_s > 0.0)))
    return fail(GAPGB_ERR_ARG, "the sigma of every fitted quantity positive, jitter non-negative");
  gapgb_status st = check_batch_host(nstruct, atom_off, lat, pos);
  if (st) return st;
  // FP64 descriptors of the training structures (the exact neighbour list)
  const int saved = m->precision;
  m->precision = GAPGB_PREC_FP64;
  double *dG = nullptr;
  st = eval_host(m, nstruct, atom_off, species, lat, pos, 0, nullptr, nullptr, nullptr, nullptr,
                 &dG);
  if (st) {
    m->precision = saved;
    return st;
  }
  const int capS = std::max(1, m->ws.h_flags[1]);  // slot count of that list
  std::vector<double> c(m->host.M);
  GAPGB_CUDA_TRY(cudaMemsetAsync(m->ws.d_flags, 0, 8 * sizeof(int), m->stream));
  st = fit_enqueue(m, nstruct, atom_off[nstruct], m->cap, capS, m->ws.d_atom_off, dG, energy,
                   forces, stress, sigma_e, sigma_f, sigma_s, jitter, c.data(), m->stream);
  m->precision = saved;
  if (st) return st;
  GAPGB_CUDA_TRY(cudaMemcpy(m->ws.h_flags, m->ws.d_flags, 8 * sizeof(int), cudaMemcpyDeviceToHost));
  st = flags_to_status(m->ws.h_flags);
  if (st) return st;
  if (coeff) std::copy(c.begin(), c.end(), coeff);
  return gapgb_model_set_coeff(m, c.data());
}

gapgb_status gapgb_fit_energies(gapgb_model *m, int nstruct, const int *atom_off,
                                const int *species, const double *lat, const double *pos,
                                const double *energy, double sigma_e, double jitter,
                                double *coeff) {
  return gapgb_fit(m, nstruct, atom_off, species, lat, pos, energy, nullptr, nullptr, sigma_e,
                   1.0, 1.0, jitter, coeff);
}

gapgb_status gapgb_model_set_qmm(gapgb_model *m, const double *qmm, int nsparse) {
  if (!m) return fail(GAPGB_ERR_ARG, "null argument");
  if (qmm && nsparse != m->host.M)
    return fail(GAPGB_ERR_ARG, "qmm must be nsparse x nsparse of the model (M = " +
                                   std::to_string(m->host.M) + ")");
  if (m->d_sf) cudaSetDevice(m->device);
  return variance_set_qmm(m, qmm);
}

gapgb_status gapgb_variance(gapgb_model *m, int nstruct, const int *atom_off, const int *species,
                            const double *lat, const double *pos, double *covf, double *variance) {
  if (!m || !atom_off || !species || !lat || !pos || !variance)
    return fail(GAPGB_ERR_ARG, "null argument");
  if (m->var.qmm.empty()) return fail(GAPGB_ERR_ARG, "no qmm attached (gapgb_model_set_qmm)");
  gapgb_status st = check_batch_host(nstruct, atom_off, lat, pos);
  if (st) return st;
  double *dG = nullptr;
  st = eval_host(m, nstruct, atom_off, species, lat, pos, 0, nullptr, nullptr, nullptr, nullptr,
                 &dG);  // neighbour list and descriptors in the model's precision
  if (st) return st;
  const int N = atom_off[nstruct];
  cudaStream_t s = m->stream;
  if (m->profile_stages) cudaEventRecord(m->ev[0], s);
  st = variance_enqueue(m, nstruct, N, m->ws.d_atom_off, dG, m->precision == GAPGB_PREC_FP64, s);
  if (st) return st;
  if (m->profile_stages) cudaEventRecord(m->ev[1], s);
  if (covf)
    GAPGB_CUDA_TRY(cudaMemcpyAsync(covf, m->var.covf, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(variance, m->var.var, sizeof(double) * nstruct,
                                 cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(m->ws.h_flags, m->ws.d_flags, 8 * sizeof(int),
                                 cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaStreamSynchronize(s));
  if (m->profile_stages) cudaEventElapsedTime(&m->var_ms, m->ev[0], m->ev[1]);
  return flags_to_status(m->ws.h_flags);
}

gapgb_status gapgb_variance_time(gapgb_model *m, float *ms) {
  if (!m || !ms) return fail(GAPGB_ERR_ARG, "null argument");
  *ms = m->var_ms;
  return GAPGB_OK;
}

gapgb_status gapgb_eval_batch(gapgb_model *m, int nstruct, const int *atom_off, const int *species,
                              const double *lat, const double *pos, int lgrad, double *energy,
                              double *force, double *stress, double *atom_energy) {
  if (!m || !atom_off || !species || !lat || !pos || !energy)
    return fail(GAPGB_ERR_ARG, "null argument");
  if (lgrad && (!force || !stress)) return fail(GAPGB_ERR_ARG, "force and stress needed with lgrad");
  return eval_host(m, nstruct, atom_off, species, lat, pos, lgrad, energy, force, stress,
                   atom_energy, nullptr);
}

gapgb_status gapgb_eval_batch_device(gapgb_model *m, int nstruct, int natoms, int max_atoms,
                                     const int *d_atom_off, const int *d_species,
                                     const double *d_lat, const double *d_pos, int lgrad,
                                     double *d_energy, double *d_force, double *d_stress,
                                     double *d_atom_energy, void *stream) {
  if (!m || !d_atom_off || !d_species || !d_lat || !d_pos || !d_energy)
    return fail(GAPGB_ERR_ARG, "null argument");
  if (nstruct <= 0 || natoms <= 0) return fail(GAPGB_ERR_ARG, "sizes must be positive");
  if (lgrad && (!d_force || !d_stress)) return fail(GAPGB_ERR_ARG, "force and stress needed with lgrad");
  gapgb_status st = upload_model(m);
  if (st) return st;
  GAPGB_CUDA_TRY(cudaSetDevice(m->device));
  st = ensure_ws(m, natoms, nstruct, m->cap);
  if (st) return st;
  if (m->precision == GAPGB_PREC_SURROGATE) {
    st = ensure_surrogate(m, natoms);
    if (st) return st;
  }
  Workspace &ws = m->ws;
  cudaStream_t s = (cudaStream_t)stream;
  const int cap = m->cap;
  GAPGB_CUDA_TRY(cudaMemsetAsync(ws.d_flags, 0, 8 * sizeof(int), s));
  if (m->profile_stages) cudaEventRecord(m->ev[0], s);
  const int maxa = max_atoms > 0 ? max_atoms : natoms;
  launch_prep(m, ws, nstruct, natoms, d_atom_off, d_species, d_lat, d_pos, m->host.rcut, s,
              maxa >= kBinMinAtoms);
  launch_neighbors(ws, nstruct, natoms, maxa, cap, m->host.rcut, s,
                   m->precision == GAPGB_PREC_FP64);
  double *d_stress_use = d_stress ? d_stress : ws.d_stress;
  double *d_force_use = d_force ? d_force : ws.d_force;
  return enqueue_tail(m, nstruct, natoms, cap, cap, lgrad, d_species, d_energy, d_force_use,
                      d_stress_use, d_atom_energy, s);
}

struct gapgb_graph {
  gapgb_model *model = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::shared_ptr<std::atomic<int>> live;  // the model's live-graph count
};

gapgb_status gapgb_graph_create(gapgb_model *m, int nstruct, int natoms, int max_atoms,
                                const int *d_atom_off, const int *d_species, const double *d_lat,
                                const double *d_pos, int lgrad, double *d_energy, double *d_force,
                                double *d_stress, double *d_atom_energy, gapgb_graph **out) {
  if (!m || !out) return fail(GAPGB_ERR_ARG, "null argument");
  *out = nullptr;
  // warm-up outside capture: workspace, tensor-core image, device flags
  gapgb_status st = gapgb_eval_batch_device(m, nstruct, natoms, max_atoms, d_atom_off, d_species,
                                            d_lat, d_pos, lgrad, d_energy, d_force, d_stress,
                                            d_atom_energy, m->stream);
  if (st) return st;
  GAPGB_CUDA_TRY(cudaStreamSynchronize(m->stream));
  st = gapgb_check_device_status(m);
  if (st) return st;
  gapgb_graph *g = new gapgb_graph();
  g->model = m;
  cudaError_t e = cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    delete g;
    return fail(GAPGB_ERR_CUDA, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e));
  }
  st = gapgb_eval_batch_device(m, nstruct, natoms, max_atoms, d_atom_off, d_species, d_lat, d_pos,
                               lgrad, d_energy, d_force, d_stress, d_atom_energy, m->stream);
  e = cudaStreamEndCapture(m->stream, &g->graph);
  if (st || e != cudaSuccess) {
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    if (st) return st;
    return fail(GAPGB_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g->graph);
    delete g;
    return fail(GAPGB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  }
  g->live = m->live_graphs;
  g->live->fetch_add(1);
  *out = g;
  return GAPGB_OK;
}

gapgb_status gapgb_graph_launch(gapgb_graph *g, void *stream) {
  if (!g || !g->exec) return fail(GAPGB_ERR_ARG, "null graph");
  GAPGB_CUDA_TRY(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  return GAPGB_OK;
}

void gapgb_graph_free(gapgb_graph *g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->live) g->live->fetch_sub(1);
  delete g;
}

gapgb_status gapgb_check_device_status(gapgb_model *m) {
  if (!m) return fail(GAPGB_ERR_ARG, "null model");
  if (!m->ws.d_flags) return GAPGB_OK;
  GAPGB_CUDA_TRY(cudaSetDevice(m->device));
  GAPGB_CUDA_TRY(cudaDeviceSynchronize());
  GAPGB_CUDA_TRY(cudaMemcpy(m->ws.h_flags, m->ws.d_flags, 8 * sizeof(int), cudaMemcpyDeviceToHost));
  read_stage_times(m);
  gapgb_status st = flags_to_status(m->ws.h_flags);
  GAPGB_CUDA_TRY(cudaMemset(m->ws.d_flags, 0, 8 * sizeof(int)));
  return st;
}

gapgb_status gapgb_stage_times(gapgb_model *m, float t[4]) {
  if (!m || !t) return fail(GAPGB_ERR_ARG, "null argument");
  for (int q = 0; q < 4; ++q) t[q] = m->stage_ms[q];
  return GAPGB_OK;
}

gapgb_status gapgb_model_set_surrogate(gapgb_model *m, gapgb_surrogate *s, double threshold_ev) {
  if (!m) return fail(GAPGB_ERR_ARG, "null model");
  if (m->live_graphs->load() > 0)
    return fail(GAPGB_ERR_ARG, "the model is bound to a live CUDA graph (free it first)");
  if (!s) {
    m->surrogate = nullptr;
    if (m->precision == GAPGB_PREC_SURROGATE) m->precision = GAPGB_PREC_MIXED;
    return GAPGB_OK;
  }
  if (!(threshold_ev >= 0.0)) return fail(GAPGB_ERR_ARG, "threshold must be >= 0");
  if (surrogate_des_len(s) != m->host.D)
    return fail(GAPGB_ERR_ARG, "surrogate des_len differs from the model's D");
  if (surrogate_device(s) != m->device)
    return fail(GAPGB_ERR_ARG, "surrogate and model live on different devices");
  for (int z : m->host.species_z)
    if (!surrogate_has_species(s, z))
      return fail(GAPGB_ERR_UNKNOWN_SPECIES, "surrogate lacks species Z=" + std::to_string(z));
  m->surrogate = s;
  m->surr_threshold = threshold_ev;
  return GAPGB_OK;
}

gapgb_status gapgb_model_set_fallback_triggers(gapgb_model *m, double grad_spread,
                                               double r_contact) {
  if (!m) return fail(GAPGB_ERR_ARG, "null model");
  if (!(grad_spread >= 0.0) || !(r_contact >= 0.0))
    return fail(GAPGB_ERR_ARG, "grad_spread and r_contact must be >= 0");
  if (m->live_graphs->load() > 0)
    return fail(GAPGB_ERR_ARG, "the model is bound to a live CUDA graph (free it first)");
  m->surr_gspread = grad_spread;
  m->surr_contact = r_contact;
  return GAPGB_OK;
}

gapgb_status gapgb_surrogate_fallback_count(gapgb_model *m, int *count) {
  if (!m || !count) return fail(GAPGB_ERR_ARG, "null argument");
  *count = 0;
  if (!m->fb_count) return GAPGB_OK;
  GAPGB_CUDA_TRY(cudaSetDevice(m->device));
  GAPGB_CUDA_TRY(cudaDeviceSynchronize());
  GAPGB_CUDA_TRY(cudaMemcpy(count, m->fb_count, sizeof(int), cudaMemcpyDeviceToHost));
  return GAPGB_OK;
}

gapgb_status gapgb_gpr_labels(gapgb_model *m, int nstruct, const int *atom_off, const int *species,
                              const double *lat, const double *pos, float *d_G, double *d_e,
                              float *d_dedg) {
  if (!m || !atom_off || !species || !lat || !pos || !d_G || !d_e || !d_dedg)
    return fail(GAPGB_ERR_ARG, "null argument");
  if (m->precision == GAPGB_PREC_SURROGATE)
    return fail(GAPGB_ERR_ARG, "labels come from the GPR: choose a GPR precision");
  gapgb_status st = check_batch_host(nstruct, atom_off, lat, pos);
  if (st) return st;
  std::vector<double> energy(nstruct);
  st = eval_host(m, nstruct, atom_off, species, lat, pos, 0, energy.data(), nullptr, nullptr,
                 nullptr, nullptr);
  if (st) return st;
  const Workspace &ws = m->ws;
  const size_t n = (size_t)atom_off[nstruct], nd = n * m->host.D;
  cudaStream_t s = m->stream;
  if (m->precision == GAPGB_PREC_FP64) {
    k_d2f<<<(unsigned)((nd + 255) / 256), 256, 0, s>>>(nd, (const double *)ws.G, d_G);
    k_d2f<<<(unsigned)((nd + 255) / 256), 256, 0, s>>>(nd, (const double *)ws.dedg, d_dedg);
  } else {
    GAPGB_CUDA_TRY(cudaMemcpyAsync(d_G, ws.G, nd * sizeof(float), cudaMemcpyDeviceToDevice, s));
    GAPGB_CUDA_TRY(cudaMemcpyAsync(d_dedg, ws.dedg, nd * sizeof(float), cudaMemcpyDeviceToDevice, s));
  }
  GAPGB_CUDA_TRY(cudaMemcpyAsync(d_e, ws.e, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  GAPGB_CUDA_TRY(cudaGetLastError());
  GAPGB_CUDA_TRY(cudaStreamSynchronize(s));
  return GAPGB_OK;
}

gapgb_status gapgb_descriptors(gapgb_model *m, int nstruct, const int *atom_off,
                               const int *species, const double *lat, const double *pos,
                               double *xx) {
  if (!m || !atom_off || !species || !lat || !pos || !xx) return fail(GAPGB_ERR_ARG, "null argument");
  const int saved = m->precision;
  m->precision = GAPGB_PREC_FP64;
  double *dG = nullptr;
  gapgb_status st = eval_host(m, nstruct, atom_off, species, lat, pos, 0, nullptr, nullptr,
                              nullptr, nullptr, &dG);
  m->precision = saved;
  if (st) return st;
  const size_t n = (size_t)atom_off[nstruct] * m->host.D;
  GAPGB_CUDA_TRY(cudaMemcpy(xx, dG, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return GAPGB_OK;
}

gapgb_status gapgb_neighbors(gapgb_model *m, int natoms, const int *species, const double *lat,
                             const double *pos, int cap, int *count, double *nb) {
  if (!m || !species || !lat || !pos || !count || !nb || natoms <= 0 || cap <= 0)
    return fail(GAPGB_ERR_ARG, "bad argument");
  const int off[2] = {0, natoms};
  gapgb_status st = check_batch_host(1, off, lat, pos);
  if (st) return st;
  st = upload_model(m);
  if (st) return st;
  GAPGB_CUDA_TRY(cudaSetDevice(m->device));
  st = ensure_ws(m, natoms, 1, cap);
  if (st) return st;
  Workspace &ws = m->ws;
  cudaStream_t s = m->stream;
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_atom_off, off, sizeof(int) * 2, cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_species, species, sizeof(int) * natoms, cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_lat, lat, sizeof(double) * 9, cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_pos, pos, sizeof(double) * 3 * natoms, cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemsetAsync(ws.d_flags, 0, 8 * sizeof(int), s));
  launch_prep(m, ws, 1, natoms, ws.d_atom_off, ws.d_species, ws.d_lat, ws.d_pos, m->host.rcut, s,
              natoms >= kBinMinAtoms);
  launch_neighbors(ws, 1, natoms, natoms, cap, m->host.rcut, s);
  GAPGB_CUDA_TRY(cudaGetLastError());
  std::vector<double4> xyz((size_t)natoms * cap);
  std::vector<int> nj((size_t)natoms * cap);
  GAPGB_CUDA_TRY(cudaMemcpyAsync(count, ws.nbr_cnt, sizeof(int) * natoms, cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(xyz.data(), ws.nbr_xyz, sizeof(double4) * xyz.size(), cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(nj.data(), ws.nbr_j, sizeof(int) * nj.size(), cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.h_flags, ws.d_flags, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaStreamSynchronize(s));
  st = flags_to_status(ws.h_flags);
  if (st) return st;
  std::vector<double> w(natoms, 0.0);
  for (int a = 0; a < natoms; ++a)
    for (int q = 0; q < m->host.nspecies; ++q)
      if (m->host.species_z[q] == species[a]) w[a] = m->host.species_w[q];
  for (int i = 0; i < natoms; ++i)
    for (int q = 0; q < count[i]; ++q) {
      const size_t k = (size_t)i * cap + q;
      double *o = nb + k * 6;
      o[0] = xyz[k].x;
      o[1] = xyz[k].y;
      o[2] = xyz[k].z;
      o[3] = xyz[k].w;
      o[4] = w[nj[k]];
      o[5] = (double)(nj[k] + 1);
    }
  return GAPGB_OK;
}

gapgb_status gapgb_min_bond(int natoms, const double *lat, const double *pos, double rcut,
                            double *min_bond) {
  if (!lat || !pos || !min_bond || natoms <= 0 || !(rcut > 0.0)) return fail(GAPGB_ERR_ARG, "bad argument");
  // a throw-away single-species model carries the workspace
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  static gapgb_model *tiny = nullptr;
  if (!tiny) {
    const int z = 0;
    const double w = 0.0, a = 0.0, c = 1.0, th = 1.0, mm2[2] = {0.0, 0.0}, co = 0.0;
    const int ty = 1;
    const double th2[2] = {th, th};
    gapgb_status st = gapgb_model_create(1, &z, &w, 1, &ty, &a, &c, nullptr, 1, 2, th2, mm2, &co,
                                         rcut, &tiny);
    if (st) return st;
  }
  tiny->host.rcut = rcut;
  std::vector<int> sp(natoms, 0);
  const int off[2] = {0, natoms};
  gapgb_status st = check_batch_host(1, off, lat, pos);
  if (st) return st;
  st = upload_model(tiny);
  if (st) return st;
  GAPGB_CUDA_TRY(cudaSetDevice(tiny->device));
  st = ensure_ws(tiny, natoms, 1, 1);
  if (st) return st;
  Workspace &ws = tiny->ws;
  cudaStream_t s = tiny->stream;
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_atom_off, off, sizeof(int) * 2, cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_species, sp.data(), sizeof(int) * natoms, cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_lat, lat, sizeof(double) * 9, cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_pos, pos, sizeof(double) * 3 * natoms, cudaMemcpyHostToDevice, s));
  GAPGB_CUDA_TRY(cudaMemsetAsync(ws.d_flags, 0, 8 * sizeof(int), s));
  const double init = 10.0;  // get_bond.f90:38
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.d_energy, &init, sizeof(double), cudaMemcpyHostToDevice, s));
  launch_prep(tiny, ws, 1, natoms, ws.d_atom_off, ws.d_species, ws.d_lat, ws.d_pos, rcut, s);
  launch_min_bond(ws, natoms, rcut, ws.d_energy, s);
  GAPGB_CUDA_TRY(cudaGetLastError());
  GAPGB_CUDA_TRY(cudaMemcpyAsync(min_bond, ws.d_energy, sizeof(double), cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaMemcpyAsync(ws.h_flags, ws.d_flags, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
  GAPGB_CUDA_TRY(cudaStreamSynchronize(s));
  if (ws.h_flags[0] & kFlagImageLimit)
    return fail(GAPGB_ERR_CAP_EXCEEDED, "more than 127 periodic images per lattice direction");
  return GAPGB_OK;
}

}  // extern "C"
