// md.cu - NVE velocity-Verlet molecular dynamics on the device.
//
// No counterpart in the reference's hot path: gappy drives MD through ASE
// with one FGAP_CALC per step (gappy/example/ASE-GAPPY/run_md.py).  Here a
// whole step - half kick + drift, (wrap,) evaluation, half kick, kinetic
// energy - is one CUDA graph launch.  Two graphs are captured: one rebuilds
// the neighbour list with cutoff rcut + skin (after wrapping the atoms into
// their cells), the other refreshes the stored slots from the current
// positions (k_nbr_refresh); a step takes the first every `rebuild_every`
// steps.  Units: Angstrom, fs, amu, eV; a = F / m * 9.648533212e-3 A/fs^2
// per eV/(A amu), KE = 1/2 m v^2 * 103.642697 eV per amu A^2/fs^2.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gapgb_internal.h"

namespace gapgb {
namespace {

constexpr double kAccel = 9.648533212331e-3;  // (eV / A / amu) in A / fs^2
constexpr double kKinetic = 103.642697;       // amu A^2 / fs^2 in eV

// v += dt/2 a, then x += dt v
__global__ void k_vv_kick_drift(int N, double *__restrict__ pos, double *__restrict__ vel,
                                const double *__restrict__ force, const double *__restrict__ accf,
                                double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double a = 0.5 * dt * accf[i];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double v = vel[3 * (size_t)i + c] + a * force[3 * (size_t)i + c];
    vel[3 * (size_t)i + c] = v;
    pos[3 * (size_t)i + c] += dt * v;
  }
}

// v += dt/2 a
__global__ void k_vv_kick(int N, double *__restrict__ vel, const double *__restrict__ force,
                          const double *__restrict__ accf, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double a = 0.5 * dt * accf[i];
#pragma unroll
  for (int c = 0; c < 3; ++c) vel[3 * (size_t)i + c] += a * force[3 * (size_t)i + c];
}

// positions into their cell: fractional f = x L^-1, f -= floor(f), x = f L
__global__ void k_md_wrap(int N, int S, const int *__restrict__ atom_off,
                          const double *__restrict__ lat, double *__restrict__ pos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int lo = 0, hi = S;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (atom_off[mid] <= i) lo = mid; else hi = mid;
  }
  const double *L = lat + (size_t)lo * 9;
  const double det = L[0] * (L[4] * L[8] - L[5] * L[7]) - L[1] * (L[3] * L[8] - L[5] * L[6]) +
                     L[2] * (L[3] * L[7] - L[4] * L[6]);
  const double inv[9] = {(L[4] * L[8] - L[5] * L[7]) / det, (L[2] * L[7] - L[1] * L[8]) / det,
                         (L[1] * L[5] - L[2] * L[4]) / det, (L[5] * L[6] - L[3] * L[8]) / det,
                         (L[0] * L[8] - L[2] * L[6]) / det, (L[2] * L[3] - L[0] * L[5]) / det,
                         (L[3] * L[7] - L[4] * L[6]) / det, (L[1] * L[6] - L[0] * L[7]) / det,
                         (L[0] * L[4] - L[1] * L[3]) / det};
  double *x = pos + 3 * (size_t)i;
  double f[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) f[a] = x[0] * inv[a] + x[1] * inv[3 + a] + x[2] * inv[6 + a];
  bool moved = false;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double fl = floor(f[a]);
    if (fl != 0.0) moved = true;
    f[a] -= fl;
  }
  if (!moved) return;  // atoms inside their cell keep their coordinates bit for bit
#pragma unroll
  for (int c = 0; c < 3; ++c) x[c] = f[0] * L[c] + f[1] * L[3 + c] + f[2] * L[6 + c];
}

// kinetic energy per structure in two fixed-order stages (parts of up to
// 64 blocks per structure, then one thread per structure)
constexpr int kKinParts = 64;

__global__ void k_md_kin_partial(int parts, const int *__restrict__ atom_off,
                                 const double *__restrict__ vel, const double *__restrict__ mass,
                                 double *__restrict__ part) {
  __shared__ double red[256];
  const int s = blockIdx.y, p = blockIdx.x;
  const int a0 = atom_off[s], na = atom_off[s + 1] - a0;
  const int len = (na + parts - 1) / parts;
  const int beg = p * len, end = min(na, beg + len);
  double acc = 0.0;
  for (int q = beg + threadIdx.x; q < end; q += blockDim.x) {
    const double *v = vel + 3 * (size_t)(a0 + q);
    acc += mass[a0 + q] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(size_t)s * parts + p] = red[0];
}

__global__ void k_md_kin_final(int S, int parts, const double *__restrict__ part,
                               double *__restrict__ ekin) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  double t = 0.0;
  for (int p = 0; p < parts; ++p) t += part[(size_t)s * parts + p];
  ekin[s] = 0.5 * kKinetic * t;
}

// displacement since the last rebuild above half the skin: flag it (the
// refreshed list could then miss a pair that came within the cutoff)
__global__ void k_md_disp(int N, const double *__restrict__ pos, const double *__restrict__ ref,
                          double half_skin2, int *__restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const double dx = pos[3 * (size_t)i] - ref[3 * (size_t)i];
  const double dy = pos[3 * (size_t)i + 1] - ref[3 * (size_t)i + 1];
  const double dz = pos[3 * (size_t)i + 2] - ref[3 * (size_t)i + 2];
  if (dx * dx + dy * dy + dz * dz > half_skin2) atomicOr(flags, kFlagSkinExceeded);
}

__global__ void k_md_accf(int N, const double *__restrict__ mass, double *__restrict__ accf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) accf[i] = kAccel / mass[i];
}

gapgb_status mfail(gapgb_status st, const std::string &msg) {
  set_last_error(msg);
  return st;
}

}  // namespace
}  // namespace gapgb

using namespace gapgb;

struct gapgb_md {
  gapgb_model *m = nullptr;
  int S = 0, N = 0, every = 10;
  double dt = 1.0, skin = 0.0;
  const int *d_atom_off = nullptr, *d_species = nullptr;
  const double *d_lat = nullptr, *d_mass = nullptr;
  double *d_pos = nullptr, *d_vel = nullptr;
  double *accf = nullptr, *energy = nullptr, *force = nullptr, *stress = nullptr, *ekin = nullptr;
  double *pos_ref = nullptr;  // positions at the last rebuild
  double *kin_part = nullptr;  // kinetic-energy partial sums [S][parts]
  int kin_parts = 1;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t g_rebuild = nullptr, g_refresh = nullptr;
  std::shared_ptr<std::atomic<int>> live;  // the model's live-graph count, once captured
  long step = 0;
};

namespace {

void kinetic(gapgb_md *md, cudaStream_t s) {
  k_md_kin_partial<<<dim3(md->kin_parts, md->S), 256, 0, s>>>(md->kin_parts, md->d_atom_off,
                                                               md->d_vel, md->d_mass, md->kin_part);
  k_md_kin_final<<<(md->S + 127) / 128, 128, 0, s>>>(md->S, md->kin_parts, md->kin_part, md->ekin);
}

// the launch sequence of one step (captured, never run directly)
gapgb_status md_step_enqueue(gapgb_md *md, bool rebuild, cudaStream_t s) {
  const unsigned b = (unsigned)((md->N + 255) / 256);
  k_vv_kick_drift<<<b, 256, 0, s>>>(md->N, md->d_pos, md->d_vel, md->force, md->accf, md->dt);
  if (rebuild) {
    k_md_wrap<<<b, 256, 0, s>>>(md->N, md->S, md->d_atom_off, md->d_lat, md->d_pos);
    GAPGB_CUDA_TRY(cudaMemcpyAsync(md->pos_ref, md->d_pos, sizeof(double) * 3 * (size_t)md->N,
                                   cudaMemcpyDeviceToDevice, s));
  } else {
    k_md_disp<<<b, 256, 0, s>>>(md->N, md->d_pos, md->pos_ref, 0.25 * md->skin * md->skin,
                                md->m->ws.d_flags);
  }
  gapgb_status st = md_eval_enqueue(md->m, md->S, md->N, md->d_atom_off, md->d_species, md->d_lat,
                                    md->d_pos, rebuild, md->skin, md->energy, md->force,
                                    md->stress, s);
  if (st) return st;
  k_vv_kick<<<b, 256, 0, s>>>(md->N, md->d_vel, md->force, md->accf, md->dt);
  kinetic(md, s);
  GAPGB_CUDA_TRY(cudaGetLastError());
  return GAPGB_OK;
}

gapgb_status capture(gapgb_md *md, bool rebuild, cudaGraphExec_t *out) {
  cudaGraph_t g = nullptr;
  GAPGB_CUDA_TRY(cudaStreamBeginCapture(md->stream, cudaStreamCaptureModeThreadLocal));
  const gapgb_status st = md_step_enqueue(md, rebuild, md->stream);
  const cudaError_t e = cudaStreamEndCapture(md->stream, &g);
  if (st) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return mfail(GAPGB_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
  const cudaError_t e2 = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e2 != cudaSuccess) return mfail(GAPGB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e2));
  return GAPGB_OK;
}

}  // namespace

extern "C" {

void gapgb_md_free(gapgb_md *md) {
  if (!md) return;
  if (md->g_rebuild) cudaGraphExecDestroy(md->g_rebuild);
  if (md->g_refresh) cudaGraphExecDestroy(md->g_refresh);
  if (md->live) md->live->fetch_sub(1);
  void *ps[] = {md->accf, md->energy, md->force, md->stress, md->ekin, md->pos_ref, md->kin_part};
  for (void *p : ps)
    if (p) cudaFree(p);
  if (md->stream) cudaStreamDestroy(md->stream);
  delete md;
}

gapgb_status gapgb_md_create(gapgb_model *m, int nstruct, int natoms, const int *d_atom_off,
                             const int *d_species, const double *d_lat, double *d_pos,
                             double *d_vel, const double *d_mass, double dt_fs, double skin,
                             int rebuild_every, gapgb_md **out) {
  if (!m || !out || !d_atom_off || !d_species || !d_lat || !d_pos || !d_vel || !d_mass)
    return mfail(GAPGB_ERR_ARG, "null argument");
  *out = nullptr;
  if (nstruct <= 0 || natoms <= 0) return mfail(GAPGB_ERR_ARG, "sizes must be positive");
  if (!(dt_fs > 0.0) || !(skin >= 0.0) || rebuild_every < 1)
    return mfail(GAPGB_ERR_ARG, "dt > 0, skin >= 0 and rebuild_every >= 1 required");
  gapgb_md *md = new gapgb_md();
  md->m = m;
  md->S = nstruct;
  md->N = natoms;
  md->dt = dt_fs;
  md->skin = skin;
  md->every = rebuild_every;
  md->d_atom_off = d_atom_off;
  md->d_species = d_species;
  md->d_lat = d_lat;
  md->d_pos = d_pos;
  md->d_vel = d_vel;
  md->d_mass = d_mass;
  md->kin_parts = std::max(1, std::min(kKinParts, natoms / nstruct / 2048));
  gapgb_status st = md_prepare(m, natoms, nstruct);
  if (st) {
    gapgb_md_free(md);
    return st;
  }
  if (cudaMalloc(&md->accf, sizeof(double) * natoms) != cudaSuccess ||
      cudaMalloc(&md->energy, sizeof(double) * nstruct) != cudaSuccess ||
      cudaMalloc(&md->force, sizeof(double) * 3 * (size_t)natoms) != cudaSuccess ||
      cudaMalloc(&md->stress, sizeof(double) * 6 * (size_t)nstruct) != cudaSuccess ||
      cudaMalloc(&md->ekin, sizeof(double) * nstruct) != cudaSuccess ||
      cudaMalloc(&md->pos_ref, sizeof(double) * 3 * (size_t)natoms) != cudaSuccess ||
      cudaMalloc(&md->kin_part, sizeof(double) * kKinParts * (size_t)nstruct) != cudaSuccess ||
      cudaStreamCreateWithFlags(&md->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    gapgb_md_free(md);
    return mfail(GAPGB_ERR_ALLOC, "MD buffers");
  }
  const unsigned b = (unsigned)((natoms + 255) / 256);
  k_md_accf<<<b, 256, 0, md->stream>>>(natoms, d_mass, md->accf);
  k_md_wrap<<<b, 256, 0, md->stream>>>(natoms, nstruct, d_atom_off, d_lat, d_pos);
  if (cudaMemcpyAsync(md->pos_ref, d_pos, sizeof(double) * 3 * (size_t)natoms,
                      cudaMemcpyDeviceToDevice, md->stream) != cudaSuccess) {
    gapgb_md_free(md);
    return mfail(GAPGB_ERR_CUDA, "MD set-up copy");
  }
  // forces at t = 0 (rebuild), growing the capacity until the list fits with
  // 25 % headroom for the rebuilds to come
  for (int attempt = 0;; ++attempt) {
    st = md_clear_flags(m);
    if (!st) st = md_eval_enqueue(m, nstruct, natoms, d_atom_off, d_species, d_lat, d_pos, true,
                                  skin, md->energy, md->force, md->stress, md->stream);
    if (!st && cudaStreamSynchronize(md->stream) != cudaSuccess)
      st = mfail(GAPGB_ERR_CUDA, std::string("MD set-up: ") + cudaGetErrorString(cudaGetLastError()));
    int maxcnt = 0;
    if (!st) st = md_read_flags(m, &maxcnt);
    const int want = ((maxcnt + maxcnt / 4 + 31) / 32) * 32;
    if ((st == GAPGB_ERR_NEIGHBOUR_OVERFLOW || (!st && want > m->cap)) && attempt < 3) {
      m->cap = want;
      st = md_prepare(m, natoms, nstruct);
      if (st) break;
      continue;
    }
    break;
  }
  if (!st) {
    kinetic(md, md->stream);
    st = capture(md, true, &md->g_rebuild);
  }
  if (!st) st = capture(md, false, &md->g_refresh);
  if (!st && cudaStreamSynchronize(md->stream) != cudaSuccess)
    st = mfail(GAPGB_ERR_CUDA, "MD set-up synchronisation");
  if (st) {
    gapgb_md_free(md);
    return st;
  }
  md->live = m->live_graphs;
  md->live->fetch_add(1);
  *out = md;
  return GAPGB_OK;
}

gapgb_status gapgb_md_run(gapgb_md *md, int nsteps, double *d_epot, double *d_ekin, void *stream) {
  if (!md || nsteps < 0) return mfail(GAPGB_ERR_ARG, "bad argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : md->stream;
  for (int k = 0; k < nsteps; ++k) {
    const long step = ++md->step;
    GAPGB_CUDA_TRY(cudaGraphLaunch(step % md->every == 0 ? md->g_rebuild : md->g_refresh, s));
    if (d_epot)
      GAPGB_CUDA_TRY(cudaMemcpyAsync(d_epot + (size_t)k * md->S, md->energy, sizeof(double) * md->S,
                                     cudaMemcpyDeviceToDevice, s));
    if (d_ekin)
      GAPGB_CUDA_TRY(cudaMemcpyAsync(d_ekin + (size_t)k * md->S, md->ekin, sizeof(double) * md->S,
                                     cudaMemcpyDeviceToDevice, s));
  }
  return GAPGB_OK;
}

gapgb_status gapgb_md_outputs(const gapgb_md *md, const double **d_energy, const double **d_force,
                              const double **d_stress, const double **d_ekin) {
  if (!md) return mfail(GAPGB_ERR_ARG, "null MD");
  if (d_energy) *d_energy = md->energy;
  if (d_force) *d_force = md->force;
  if (d_stress) *d_stress = md->stress;
  if (d_ekin) *d_ekin = md->ekin;
  return GAPGB_OK;
}

gapgb_status gapgb_md_check(gapgb_md *md) {
  if (!md) return mfail(GAPGB_ERR_ARG, "null MD");
  GAPGB_CUDA_TRY(cudaSetDevice(md->m->device));
  GAPGB_CUDA_TRY(cudaDeviceSynchronize());
  const gapgb_status st = md_read_flags(md->m, nullptr);
  md_clear_flags(md->m);
  return st;
}

}  // extern "C"
