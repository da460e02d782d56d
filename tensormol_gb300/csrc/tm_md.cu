// Device-resident FP64 integrators consuming the energy/force path.
//
// Reference (Simulations/SimpleMD.py):
//   VelocityVerletStep :14-38   x += v dt + a dt^2/2; a' = 1e-10 F/m; v += (a + a') dt/2
//   KineticEnergy      :40-51   per-atom KE in J/mol
//   NoseThermostat     :104-129 Q = kT (20 dt N)^2, DOF term (3N+1)/2
//   NoseChainThermostat:206-320 Martyna et al. (1996) chain, nc = 2, ny = 3
//     Suzuki-Yoshida weights, Q0 = 3 N kT tau^2, Qi = kT tau^2, tau = 80 dt.
//     The chain is integrated as in the paper (particle velocities scaled by
//     the first chain element; SimpleMD.py:304 uses the second one, and its
//     step() cannot run as written, SimpleMD.py:220/277).
// Masses in kg/mol (PhysicalData.py:57), velocities A/fs, forces J/mol/A.
// Every step runs on the device without a host round trip: reductions are
// two-level and deterministic, thermostat scalars live in device memory.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "tm_internal.h"

int tm_energy_force_device(tm_system* s, unsigned flags);

namespace {
constexpr int RB = 256;   // reduction blocks
constexpr double kJph = 2625.499638 * 1000.0;
constexpr double kR = 8.3144621;

// device scalars
enum {
  S_KE2 = 0,      // sum m v^2 of the current velocities
  S_KE2B,         // second KE buffer (Nose half-step velocities)
  S_ETA,          // Nose eta
  S_XI,           // Nose integral of eta (for the conserved quantity)
  S_SCALE,        // NHC velocity scale of the last half-step
  S_CHAIN,        // NHC: eta[M], veta[M], G[M], Q[M] from here
};

__global__ void k_sum_mv2(const double* __restrict__ v, const double* __restrict__ m, int N,
                          double* __restrict__ part) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    acc += m[i] * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_sum_final(const double* __restrict__ part, int n, double* __restrict__ dst) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *dst = sh[0];
}

__global__ void k_vv_pos(double* __restrict__ x, const double* __restrict__ v,
                         const double* __restrict__ a, double dt, int n3) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n3) x[q] = x[q] + v[q] * dt + 0.5 * a[q] * dt * dt;
}

__global__ void k_vv_vel(double* __restrict__ v, double* __restrict__ a, const double* __restrict__ F,
                         const double* __restrict__ m, double dt, int n3) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n3) return;
  const double an = 1e-10 * F[q] / m[q / 3];
  v[q] = v[q] + 0.5 * (a[q] + an) * dt;
  a[q] = an;
}

// Positions into the cell (ModuloLattice, Periodic.py:87-100): orthorhombic
// cells per axis, others through fractional coordinates f = x B^-1, f - floor(f).
__global__ void k_wrap(double* __restrict__ x, const tm_mat3 lat, const tm_mat3 binv, int ortho,
                       int N) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (ortho) {
    const double L[3] = {lat.v[0], lat.v[4], lat.v[8]};
    for (int d = 0; d < 3; ++d) {
      double v = x[3 * i + d];
      v = v - L[d] * floor(v / L[d]);
      if (v >= L[d]) v -= L[d];
      x[3 * i + d] = v;
    }
    return;
  }
  const double p[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
  double f[3];
  for (int d = 0; d < 3; ++d) {
    f[d] = p[0] * binv.v[d] + p[1] * binv.v[3 + d] + p[2] * binv.v[6 + d];
    f[d] -= floor(f[d]);
    if (f[d] >= 1.0) f[d] -= 1.0;
  }
  for (int d = 0; d < 3; ++d) x[3 * i + d] = f[0] * lat.v[d] + f[1] * lat.v[3 + d] + f[2] * lat.v[6 + d];
}

// Nose: x, v(dt/2) (SimpleMD.py:117-118)
__global__ void k_nose_pos(double* __restrict__ x, const double* __restrict__ v,
                           const double* __restrict__ a, double* __restrict__ vh,
                           const double* __restrict__ sc, double dt, int n3) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n3) return;
  const double eta = sc[S_ETA];
  x[q] = x[q] + v[q] * dt + 0.5 * (a[q] - eta * v[q]) * dt * dt;
  vh[q] = v[q] + 0.5 * (a[q] - eta * v[q]) * dt;
}

// Nose eta update (SimpleMD.py:124-126); ke uses the pre-step velocities
__global__ void k_nose_eta(double* __restrict__ sc, double Q, double kT, double N, double dt) {
  const double ke = 0.5 * sc[S_KE2], kedto2 = 0.5 * sc[S_KE2B];
  const double dof = (3.0 * N + 1.0) / 2.0;
  const double e0 = sc[S_ETA];
  const double etadto2 = e0 + (dt / (2.0 * Q)) * (ke - dof * kT);
  const double e1 = etadto2 + (dt / (2.0 * Q)) * (kedto2 - dof * kT);
  sc[S_XI] += 0.5 * (e0 + e1) * dt;
  sc[S_ETA] = e1;
}

__global__ void k_nose_vel(double* __restrict__ v, double* __restrict__ a,
                           const double* __restrict__ vh, const double* __restrict__ F,
                           const double* __restrict__ m, const double* __restrict__ sc, double dt,
                           int n3) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n3) return;
  const double an = 1e-10 * F[q] / m[q / 3];
  v[q] = (vh[q] + (dt / 2.0) * an) / (1.0 + (dt / 2.0) * sc[S_ETA]);
  a[q] = an;
}

// One chain half-step (Martyna et al. 1996, Appendix A); writes the
// velocity scale to sc[S_SCALE]. Single thread: M is 1-10.
__global__ void k_nhc_chain(double* __restrict__ sc, int M, double kT, double gnkt, double dt) {
  double* eta = sc + S_CHAIN;
  double* veta = eta + M;
  double* G = veta + M;
  const double* Q = G + M;
  const double ake2 = sc[S_KE2];
  const double w = 1.0 / (2.0 - pow(2.0, 1.0 / 3.0));
  const double wj[3] = {w, 1.0 - 2.0 * w, w};
  const int nc = 2;
  G[0] = (ake2 - gnkt) / Q[0];
  for (int i = 0; i + 1 < M; ++i) G[i + 1] = (Q[i] * veta[i] * veta[i] - kT) / Q[i + 1];
  double scale = 1.0;
  for (int c = 0; c < nc; ++c) {
    for (int j = 0; j < 3; ++j) {
      const double d2 = (wj[j] * dt / nc) / 2.0, d4 = d2 / 2.0, d8 = d2 / 4.0;
      veta[M - 1] += G[M - 1] * d4;
      for (int i = M - 2; i >= 0; --i) {
        const double aa = exp(-d8 * veta[i + 1]);
        veta[i] = veta[i] * aa * aa + d4 * G[i] * aa;
      }
      const double aa = exp(-d2 * veta[0]);
      scale *= aa;
      G[0] = (scale * scale * ake2 - gnkt) / Q[0];
      for (int i = 0; i < M; ++i) eta[i] += veta[i] * d2;
      for (int i = 0; i + 1 < M; ++i) {
        const double bb = exp(-d8 * veta[i + 1]);
        veta[i] = veta[i] * bb * bb + d4 * G[i] * bb;
        G[i + 1] = (Q[i] * veta[i] * veta[i] - kT) / Q[i + 1];
      }
      veta[M - 1] += G[M - 1] * d4;
    }
  }
  sc[S_SCALE] = scale;
}

__global__ void k_scale(double* __restrict__ v, const double* __restrict__ sc, int n3) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n3) v[q] *= sc[S_SCALE];
}

__global__ void k_kick(double* __restrict__ v, const double* __restrict__ a, double h, int n3) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n3) v[q] += h * a[q];
}

__global__ void k_drift(double* __restrict__ x, const double* __restrict__ v, double dt, int n3) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n3) x[q] += dt * v[q];
}

__global__ void k_accel(double* __restrict__ a, const double* __restrict__ F,
                        const double* __restrict__ m, int n3) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n3) a[q] = 1e-10 * F[q] / m[q / 3];
}

// log row: potential (Hartree, summed over molecules), KE per atom (J/mol),
// conserved (J/mol), T_eff (K)
// The row is log + 4 * (*step); the step counter lives on the device so that
// one captured step can be replayed.
__global__ void k_log(double* __restrict__ log, int* __restrict__ step,
                      const double* __restrict__ molE, int nmol,
                      const double* __restrict__ sc, int kind, int M, double kT, double gnkt,
                      double Qnose, double N) {
  double* row = log + 4 * (size_t)(*step);
  *step += 1;
  double pe = 0.0;
  for (int m = 0; m < nmol; ++m) pe += molE[4 * m];
  const double ke = 0.5 * sc[S_KE2] * 1e10;   // J/mol total
  double cons = ke + pe * kJph;
  if (kind == TM_MD_NOSE) {
    const double eta = sc[S_ETA];
    cons += (0.5 * Qnose * eta * eta + (3.0 * N + 1.0) * kT * sc[S_XI]) * 1e10;
  } else if (kind == TM_MD_NHC) {
    const double* eta = sc + S_CHAIN;
    const double* veta = eta + M;
    const double* Q = veta + 2 * M;
    double ch = gnkt * eta[0];
    for (int i = 0; i < M; ++i) ch += 0.5 * Q[i] * veta[i] * veta[i];
    for (int i = 1; i < M; ++i) ch += kT * eta[i];
    cons += ch * 1e10;
  }
  row[0] = pe;
  row[1] = ke / N;
  row[2] = cons;
  row[3] = (2.0 / 3.0) * (ke / N) / kR;
}

}  // namespace

struct tm_md {
  tm_system* s = nullptr;
  int kind = 0, M = 0;
  double dt = 0, T = 0, kT = 0, gnkt = 0, Qnose = 0;
  double* v = nullptr;
  double* a = nullptr;
  double* m = nullptr;
  double* vh = nullptr;
  double* sc = nullptr;
  double* part = nullptr;
  double* ck_x = nullptr;    // chunk-start copies (overflow replay)
  double* ck_v = nullptr;
  double* ck_a = nullptr;
  double* ck_sc = nullptr;
  size_t bytes = 0;
};

static const double kMassAmu[11] = {0, 1.00794, 4.002602, 6.941, 9.012182, 10.811, 12.0107,
                                    14.0067, 15.9994, 18.9984032, 20.1791};

extern "C" int tm_md_create(tm_system* s, int kind, double dt, double T, int chain, tm_md** out) {
  *out = nullptr;
  if (!s || dt <= 0 || T < 0) return TM_E_ARG;
  tm_ctx* ctx = s->ctx;
  if (kind < TM_MD_NVE || kind > TM_MD_NHC) return tm_fail(ctx, TM_E_ARG, "md kind");
  // a cell below twice the cutoff is evaluated as a supercell whose copies
  // would drift apart in a trajectory (their FP32 sums run in different orders)
  if (s->K > 1) return tm_fail(ctx, TM_E_UNSUPPORTED, "MD of a cell below twice the cutoff");
  if (kind == TM_MD_NHC && (chain < 1 || chain > 10)) return tm_fail(ctx, TM_E_ARG, "chain length 1..10");
  tm_md* md = new tm_md();
  md->s = s;
  md->kind = kind;
  md->M = kind == TM_MD_NHC ? chain : 0;
  md->dt = dt;
  md->T = T;
  md->kT = kR * 1e-10 * T;                 // kg/mol (A/fs)^2
  const int N = s->N;
  md->gnkt = 3.0 * N * md->kT;
  md->Qnose = md->kT * (20.0 * dt * N) * (20.0 * dt * N);
  const size_t n3 = (size_t)3 * N;
  const size_t nsc = S_CHAIN + 4 * 10;
  int rc;
  if ((rc = tm_alloc(ctx, (void**)&md->v, n3 * 8)) || (rc = tm_alloc(ctx, (void**)&md->a, n3 * 8)) ||
      (rc = tm_alloc(ctx, (void**)&md->vh, n3 * 8)) || (rc = tm_alloc(ctx, (void**)&md->m, (size_t)N * 8)) ||
      (rc = tm_alloc(ctx, (void**)&md->sc, nsc * 8)) || (rc = tm_alloc(ctx, (void**)&md->part, RB * 8)) ||
      (rc = tm_alloc(ctx, (void**)&md->ck_x, n3 * 8)) || (rc = tm_alloc(ctx, (void**)&md->ck_v, n3 * 8)) ||
      (rc = tm_alloc(ctx, (void**)&md->ck_a, n3 * 8)) || (rc = tm_alloc(ctx, (void**)&md->ck_sc, nsc * 8))) {
    delete md;
    return rc;
  }
  std::vector<double> mass(N);
  for (int i = 0; i < N; ++i) mass[i] = 0.000999977 * kMassAmu[s->Z[i]];
  std::vector<double> sc(nsc, 0.0);
  sc[S_SCALE] = 1.0;
  if (kind == TM_MD_NHC) {
    const double tau = 80.0 * dt;
    double* Q = sc.data() + S_CHAIN + 3 * md->M;
    for (int i = 0; i < md->M; ++i) Q[i] = md->kT * tau * tau;
    Q[0] = 3.0 * N * md->kT * tau * tau;
  }
  cudaStream_t st = ctx->stream;
  cudaMemsetAsync(md->v, 0, n3 * 8, st);
  cudaMemsetAsync(md->a, 0, n3 * 8, st);   // SimpleMD.py:359: the first acceleration is zero
  cudaMemcpyAsync(md->m, mass.data(), (size_t)N * 8, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(md->sc, sc.data(), nsc * 8, cudaMemcpyHostToDevice, st);
  if ((rc = tm_cuda_check(ctx, cudaStreamSynchronize(st), "md create"))) {
    delete md;
    return rc;
  }
  *out = md;
  return TM_OK;
}

extern "C" int tm_md_destroy(tm_md* md) {
  if (!md) return TM_OK;
  tm_ctx* ctx = md->s->ctx;
  const size_t n3 = (size_t)3 * md->s->N;
  tm_free(ctx, md->v, n3 * 8);
  tm_free(ctx, md->a, n3 * 8);
  tm_free(ctx, md->vh, n3 * 8);
  tm_free(ctx, md->m, (size_t)md->s->N * 8);
  tm_free(ctx, md->sc, (S_CHAIN + 40) * 8);
  tm_free(ctx, md->part, RB * 8);
  tm_free(ctx, md->ck_x, n3 * 8);
  tm_free(ctx, md->ck_v, n3 * 8);
  tm_free(ctx, md->ck_a, n3 * 8);
  tm_free(ctx, md->ck_sc, (S_CHAIN + 40) * 8);
  cudaStreamSynchronize(ctx->stream);
  delete md;
  return TM_OK;
}

extern "C" int tm_md_set_velocities(tm_md* md, const double* v, int on_device) {
  if (!md || !v) return TM_E_ARG;
  tm_ctx* ctx = md->s->ctx;
  return tm_cuda_check(ctx, cudaMemcpyAsync(md->v, v, sizeof(double) * 3 * md->s->N,
                                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                            ctx->stream),
                       "velocities");
}

extern "C" int tm_md_get_velocities(tm_md* md, double* v, int on_device) {
  if (!md || !v) return TM_E_ARG;
  tm_ctx* ctx = md->s->ctx;
  int rc = tm_cuda_check(ctx, cudaMemcpyAsync(v, md->v, sizeof(double) * 3 * md->s->N,
                                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                              ctx->stream),
                         "velocities");
  if (rc) return rc;
  return tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "velocities");
}

static void ke_into(tm_md* md, const double* v, int slot) {
  tm_ctx* ctx = md->s->ctx;
  k_sum_mv2<<<RB, 256, 0, ctx->stream>>>(v, md->m, md->s->N, md->part);
  k_sum_final<<<1, 256, 0, ctx->stream>>>(md->part, RB, md->sc + slot);
  ctx->launches += 2;
}

// One integrator step (all kernels enqueued, no host synchronisation).
static int md_step(tm_md* md, double* dlog, int* dstep) {
  tm_system* s = md->s;
  tm_ctx* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  const int N = s->N, n3 = 3 * N;
  const int gb = tm_div_up(n3, 256);
  const double dt = md->dt;
  const unsigned flags = 0;
  // periodic positions go back into the cell at every full list build; with
  // skin lists they stay continuous between candidate builds (a candidate's
  // image code refers to the positions it was built from)
  const bool wrap = s->periodic && !(s->skin > 0.0 && s->cand_valid && !s->cand_rebuild);
  int rc;
  if (md->kind == TM_MD_NVE) {
    k_vv_pos<<<gb, 256, 0, st>>>(s->d_x, md->v, md->a, dt, n3);
    ctx->launches++;
    if (wrap) { k_wrap<<<tm_div_up(N, 256), 256, 0, st>>>(s->d_x, tm_mat3_of(s->lat), tm_mat3_of(s->binv), s->ortho, N); ctx->launches++; }
    if ((rc = tm_energy_force_device(s, flags))) return rc;
    k_vv_vel<<<gb, 256, 0, st>>>(md->v, md->a, s->d_F, md->m, dt, n3);
    ctx->launches++;
    ke_into(md, md->v, S_KE2);
  } else if (md->kind == TM_MD_NOSE) {
    ke_into(md, md->v, S_KE2);
    k_nose_pos<<<gb, 256, 0, st>>>(s->d_x, md->v, md->a, md->vh, md->sc, dt, n3);
    ctx->launches++;
    if (wrap) { k_wrap<<<tm_div_up(N, 256), 256, 0, st>>>(s->d_x, tm_mat3_of(s->lat), tm_mat3_of(s->binv), s->ortho, N); ctx->launches++; }
    ke_into(md, md->vh, S_KE2B);
    if ((rc = tm_energy_force_device(s, flags))) return rc;
    k_nose_eta<<<1, 1, 0, st>>>(md->sc, md->Qnose, md->kT, (double)N, dt);
    k_nose_vel<<<gb, 256, 0, st>>>(md->v, md->a, md->vh, s->d_F, md->m, md->sc, dt, n3);
    ctx->launches += 2;
    ke_into(md, md->v, S_KE2);
  } else {
    ke_into(md, md->v, S_KE2);
    k_nhc_chain<<<1, 1, 0, st>>>(md->sc, md->M, md->kT, md->gnkt, dt);
    k_scale<<<gb, 256, 0, st>>>(md->v, md->sc, n3);
    k_kick<<<gb, 256, 0, st>>>(md->v, md->a, 0.5 * dt, n3);
    k_drift<<<gb, 256, 0, st>>>(s->d_x, md->v, dt, n3);
    ctx->launches += 4;
    if (wrap) { k_wrap<<<tm_div_up(N, 256), 256, 0, st>>>(s->d_x, tm_mat3_of(s->lat), tm_mat3_of(s->binv), s->ortho, N); ctx->launches++; }
    if ((rc = tm_energy_force_device(s, flags))) return rc;
    k_accel<<<gb, 256, 0, st>>>(md->a, s->d_F, md->m, n3);
    k_kick<<<gb, 256, 0, st>>>(md->v, md->a, 0.5 * dt, n3);
    ctx->launches += 2;
    ke_into(md, md->v, S_KE2);
    k_nhc_chain<<<1, 1, 0, st>>>(md->sc, md->M, md->kT, md->gnkt, dt);
    k_scale<<<gb, 256, 0, st>>>(md->v, md->sc, n3);
    ctx->launches += 2;
    ke_into(md, md->v, S_KE2);
  }
  k_log<<<1, 1, 0, st>>>(dlog, dstep, s->d_mol_E, s->nmol, md->sc, md->kind, md->M, md->kT,
                         md->gnkt, md->Qnose, (double)N);
  ctx->launches++;
  return TM_OK;
}

// Steps run in chunks. Each chunk starts from a device-side copy of the state
// (positions, velocities, accelerations, thermostat scalars); the
// neighbour-row overflow counters stay armed across the chunk's list builds.
// If any build of the chunk overflowed its rows, the rows are grown and the
// chunk is run again from the copy, so a run never keeps a force computed
// from a truncated row. One host synchronisation per chunk. Within a chunk the
// launch sequence of one step is captured once into a CUDA graph and replayed;
// it is captured again after buffers are replaced.
// skin > 0: the first step of every chunk builds candidate lists within the
// cutoffs + skin and the other steps filter them (exact rows every step). The
// chunk length adapts so that no atom moves more than skin/2 within a chunk
// (estimated from the largest displacement seen in the previous chunk); a chunk
// that exceeded it anyway is run again from its copy, shorter.
extern "C" int tm_md_run(tm_md* md, int nsteps, double skin, double* log) {
  if (!md || nsteps < 0 || !(skin >= 0)) return TM_E_ARG;
  tm_system* s = md->s;
  tm_ctx* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  const size_t n3b = sizeof(double) * 3 * (size_t)s->N;
  const size_t nsc = sizeof(double) * (S_CHAIN + 40);
  constexpr int kChunk = 64;
  double* dlog = nullptr;
  int* dstep = nullptr;
  int rc = TM_OK;
  if (nsteps == 0) return TM_OK;
  if ((rc = tm_alloc(ctx, (void**)&dlog, sizeof(double) * 4 * nsteps)) ||
      (rc = tm_alloc(ctx, (void**)&dstep, sizeof(int))))
    return rc;
  s->need_sticky = true;
  s->skin = skin;
  s->cand_valid = false;
  cudaGraphExec_t exec = nullptr;
  int64_t launches_per_step = 0;
  int start = 0, retries = 0;
  int chunk = skin > 0.0 ? 8 : kChunk;
  while (!rc && start < nsteps) {
    const int n = nsteps - start < chunk ? nsteps - start : chunk;
    cudaMemcpyAsync(md->ck_x, s->d_x, n3b, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(md->ck_v, md->v, n3b, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(md->ck_a, md->a, n3b, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(md->ck_sc, md->sc, nsc, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(s->d_need, 0, sizeof(int32_t) * 2, st);
    cudaMemsetAsync(s->d_need_c, 0, sizeof(int32_t) * 2, st);
    cudaMemcpyAsync(dstep, &start, sizeof(int), cudaMemcpyHostToDevice, st);
    // first step of the chunk, uncaptured: a full build (candidates when skin > 0)
    s->cand_rebuild = true;
    const int64_t l0 = ctx->launches;
    rc = md_step(md, dlog, dstep);
    const int64_t first_launches = ctx->launches - l0;
    int q = 1;
    if (!rc && !exec && q < n) {
      cudaGraph_t graph = nullptr;
      cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        const int64_t l1 = ctx->launches;
        rc = md_step(md, dlog, dstep);
        launches_per_step = ctx->launches - l1;
        ctx->launches = l1;
        e = cudaStreamEndCapture(st, &graph);
        if (!rc && e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
      }
      if (!rc && e != cudaSuccess) rc = tm_cuda_check(ctx, e, "md step graph");
    }
    (void)first_launches;
    for (; q < n && !rc; ++q) {
      rc = tm_cuda_check(ctx, cudaGraphLaunch(exec, st), "md step replay");
      ctx->launches += launches_per_step;
    }
    if (rc) break;
    unsigned long long disp_bits = 0;
    int32_t need_c[2] = {0, 0};
    if (skin > 0.0) {
      cudaMemcpyAsync(&disp_bits, s->d_disp, sizeof(disp_bits), cudaMemcpyDeviceToHost, st);
      cudaMemcpyAsync(need_c, s->d_need_c, sizeof(need_c), cudaMemcpyDeviceToHost, st);
    }
    bool grew = false;
    if ((rc = tm_nlist_grow(s, &grew))) break;          // synchronises the stream
    if ((rc = tm_sync_status(ctx, "md chunk"))) break;  // a device error ends the run
    double disp = 0.0;
    memcpy(&disp, &disp_bits, sizeof(disp));
    disp = sqrt(disp);
    bool replay = grew;
    if (skin > 0.0 && need_c[0] > s->KC) {              // candidate rows too short
      const int KC = ((need_c[0] + 31) / 32) * 32;
      tm_free(ctx, s->d_cand, sizeof(uint32_t) * (size_t)s->N_cap * s->KC);
      s->bytes -= sizeof(uint32_t) * (size_t)s->N_cap * s->KC;
      s->KC = KC;
      if ((rc = tm_alloc(ctx, (void**)&s->d_cand, sizeof(uint32_t) * (size_t)s->N_cap * KC))) break;
      s->bytes += sizeof(uint32_t) * (size_t)s->N_cap * KC;
      replay = true;
    }
    if (skin > 0.0 && disp > 0.5 * skin) {               // moved too far for the candidates
      chunk = chunk > 1 ? chunk / 2 : 1;
      replay = true;
    }
    if (replay) {
      if (++retries > 16) { rc = tm_fail(ctx, TM_E_CAPACITY, "MD chunk cannot be completed"); break; }
      cudaMemcpyAsync(s->d_x, md->ck_x, n3b, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(md->v, md->ck_v, n3b, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(md->a, md->ck_a, n3b, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(md->sc, md->ck_sc, nsc, cudaMemcpyDeviceToDevice, st);
      if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }   // buffers may be new
      continue;                                          // the same chunk again
    }
    if (skin > 0.0) {
      // the next chunk: as long as the last one's displacement, scaled, allows
      // (a one-step chunk measures no displacement), and at most twice as long
      const double per_step = disp / (n > 1 ? n - 1 : 1);
      int next = per_step > 0 ? (int)floor(0.5 * skin / (1.3 * per_step)) + 1 : kChunk;
      if (next > 2 * n) next = 2 * n;
      chunk = next < 1 ? 1 : (next > kChunk ? kChunk : next);
    }
    start += n;
    retries = 0;   // the replay limit is per chunk
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (!rc && s->periodic && skin > 0.0) {   // hand back positions inside the cell
    k_wrap<<<tm_div_up(s->N, 256), 256, 0, st>>>(s->d_x, tm_mat3_of(s->lat), tm_mat3_of(s->binv), s->ortho, s->N);
    ctx->launches++;
  }
  s->need_sticky = false;
  s->skin = 0.0;
  s->cand_valid = false;
  s->cand_rebuild = true;
  s->nlist_valid = false;
  if (!rc && log)
    rc = tm_cuda_check(ctx, cudaMemcpyAsync(log, dlog, sizeof(double) * 4 * nsteps, cudaMemcpyDeviceToHost, st), "md log");
  tm_free(ctx, dlog, sizeof(double) * 4 * nsteps);
  tm_free(ctx, dstep, sizeof(int));
  if (!rc) rc = tm_sync_status(ctx, "md_run");
  return rc;
}
