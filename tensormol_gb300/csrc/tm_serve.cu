// Continuous-batching serving state.
//
// One capacity-sized system holds every request in flight as one molecule of a
// ragged batch; a step is one fused energy+force evaluation of the whole batch
// plus, for molecular-dynamics requests, the velocity-Verlet update
// (Simulations/SimpleMD.py:14-38; the first acceleration of a new request is
// zero, as VelocityVerlet.__init__ sets it, :359). Requests join and leave
// between steps: tm_serve_layout gathers the positions, velocities and
// accelerations of the requests that stay into the new order on the device and
// appends the new ones, so nothing that is in flight goes through the host.
// Optimisation requests relax by FIRE (Bitzek, Koskinen, Gaehler, Moseler and
// Gumbsch, Phys. Rev. Lett. 97, 170201 (2006)): semi-implicit Euler steps with
// the mixing v <- (1 - alpha) v + alpha |v| F/|F|, the step growing (x1.1, up
// to 8 dt) and alpha shrinking (x0.99) after 5 downhill steps, and v = 0,
// step x0.5, alpha = 0.1 when F.v < 0; no atom moves more than 0.2 A in a
// step; per-molecule sums are two-level and deterministic.
// Molecules are independent in every kernel (per-molecule cell grids, element
// rows that never mix atoms within a row, per-molecule chunked reductions), so
// a request's results do not depend on what else is in the batch.
#include <cuda_runtime.h>

#include <vector>

#include <algorithm>

#include "tm_internal.h"

struct tm_serve {
  tm_system* s = nullptr;
  tm_ctx* ctx = nullptr;
  double dt = 0.5;
  double* v = nullptr;     // [N_cap][3] A/fs
  double* a = nullptr;     // [N_cap][3] A/fs^2
  double* m = nullptr;     // [N_cap] kg/mol
  double* x2 = nullptr;    // relayout targets (swapped with the live arrays)
  double* v2 = nullptr;
  double* a2 = nullptr;
  int32_t* src = nullptr;  // [N_cap] previous index, or -(k+1) for new row k
  double* xnew = nullptr;  // [N_cap][3] packed new rows
  double* vnew = nullptr;
  int32_t* mode = nullptr; // [nmol_cap] TM_SERVE_EF / TM_SERVE_MD / TM_SERVE_OPT
  // FIRE state per molecule (optimisation requests), and its relayout copies
  double* fire = nullptr;   // [nmol_cap][2]: dt (fs), alpha
  int32_t* npos = nullptr;  // [nmol_cap] steps since the last uphill move
  double* fire2 = nullptr;
  int32_t* npos2 = nullptr;
  int32_t* msrc = nullptr;  // [nmol_cap] previous molecule of each new molecule, or -1
  double* fmax = nullptr;   // [nmol_cap] largest |F| per molecule (J/mol/A)
  double* coef = nullptr;   // [nmol_cap][3] per-step FIRE coefficients
  size_t bytes = 0;
};

namespace {

constexpr double kFireAlpha0 = 0.1;
constexpr int kFireNmin = 5;
constexpr double kFireDtMax = 8.0;   // largest FIRE step, in units of the serving dt
constexpr double kFireMaxMove = 0.2; // A per atom and step

__constant__ double c_mass_amu[11] = {0, 1.00794, 4.002602, 6.941, 9.012182, 10.811, 12.0107,
                                      14.0067, 15.9994, 18.9984032, 20.1791};

__global__ void k_serve_gather(const int32_t* __restrict__ src, int N, const double* __restrict__ x,
                               const double* __restrict__ v, const double* __restrict__ a,
                               const double* __restrict__ xnew, const double* __restrict__ vnew,
                               const int32_t* __restrict__ Z, double* __restrict__ x2,
                               double* __restrict__ v2, double* __restrict__ a2,
                               double* __restrict__ m) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int s = src[i];
  for (int d = 0; d < 3; ++d) {
    if (s >= 0) {
      x2[3 * i + d] = x[3 * s + d];
      v2[3 * i + d] = v[3 * s + d];
      a2[3 * i + d] = a[3 * s + d];
    } else {
      const int k = -s - 1;
      x2[3 * i + d] = xnew[3 * k + d];
      v2[3 * i + d] = vnew[3 * k + d];
      a2[3 * i + d] = 0.0;
    }
  }
  const int z = Z[i];
  m[i] = 0.000999977 * c_mass_amu[(z >= 1 && z <= 10) ? z : 0];   // PhysicalData.py:57
}

// x += v dt + a dt^2 / 2 for atoms of molecular-dynamics requests
__global__ void k_serve_pre(double* __restrict__ x, const double* __restrict__ v,
                            const double* __restrict__ a, const int32_t* __restrict__ mol,
                            const int32_t* __restrict__ mode, double dt, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || mode[mol[i]] != TM_SERVE_MD) return;
  for (int d = 0; d < 3; ++d)
    x[3 * i + d] = x[3 * i + d] + v[3 * i + d] * dt + 0.5 * a[3 * i + d] * dt * dt;
}

// a' = 1e-10 F / m; v += (a + a') dt / 2; a = a'
__global__ void k_serve_post(double* __restrict__ v, double* __restrict__ a,
                             const double* __restrict__ F, const double* __restrict__ m,
                             const int32_t* __restrict__ mol, const int32_t* __restrict__ mode,
                             double dt, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || mode[mol[i]] != TM_SERVE_MD) return;
  for (int d = 0; d < 3; ++d) {
    const double an = 1e-10 * F[3 * i + d] / m[i];
    v[3 * i + d] = v[3 * i + d] + 0.5 * (a[3 * i + d] + an) * dt;
    a[3 * i + d] = an;
  }
}

// molecule state carried across a relayout; new molecules start fresh
__global__ void k_fire_gather(const int32_t* __restrict__ msrc, int nmol, const double* __restrict__ f,
                              const int32_t* __restrict__ np, double* __restrict__ f2,
                              int32_t* __restrict__ np2, double dt0) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nmol) return;
  const int o = msrc[q];
  f2[2 * q] = o >= 0 ? f[2 * o] : dt0;
  f2[2 * q + 1] = o >= 0 ? f[2 * o + 1] : kFireAlpha0;
  np2[q] = o >= 0 ? np[o] : 0;
}

// per chunk (<= TM_CHUNK atoms of one molecule): F.v, F.F, v.v, max |F|^2
__global__ void k_fire_chunk(const int2* __restrict__ chunk, const int32_t* __restrict__ mol,
                             const int32_t* __restrict__ mode, const double* __restrict__ F,
                             const double* __restrict__ v, double* __restrict__ part) {
  const int2 ch = chunk[blockIdx.x];
  __shared__ double sh[4][256];
  double fv = 0, ff = 0, vv = 0, fm = 0;
  const bool opt = mode[mol[ch.x]] == TM_SERVE_OPT;
  for (int i = ch.x + threadIdx.x; opt && i < ch.y; i += blockDim.x) {
    double f2 = 0;
    for (int d = 0; d < 3; ++d) {
      const double fd = F[3 * i + d], vd = v[3 * i + d];
      fv += fd * vd;
      f2 += fd * fd;
      vv += vd * vd;
    }
    ff += f2;
    fm = fmax(fm, f2);
  }
  sh[0][threadIdx.x] = fv;
  sh[1][threadIdx.x] = ff;
  sh[2][threadIdx.x] = vv;
  sh[3][threadIdx.x] = fm;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + o];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + o];
      sh[2][threadIdx.x] += sh[2][threadIdx.x + o];
      sh[3][threadIdx.x] = fmax(sh[3][threadIdx.x], sh[3][threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) part[8 * (size_t)blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

// per molecule: FIRE decisions; coef[q] = (cv, cf, dt) for the atom update
__global__ void k_fire_mol(const int32_t* __restrict__ mol_chunk, const double* __restrict__ part,
                           const int32_t* __restrict__ mode, double* __restrict__ f,
                           int32_t* __restrict__ np, double* __restrict__ coef,
                           double* __restrict__ fmaxo, int nmol, double dtmax) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nmol) return;
  double fv = 0, ff = 0, vv = 0, fm = 0;
  for (int c = mol_chunk[q]; c < mol_chunk[q + 1]; ++c) {
    fv += part[8 * (size_t)c];
    ff += part[8 * (size_t)c + 1];
    vv += part[8 * (size_t)c + 2];
    fm = fmax(fm, part[8 * (size_t)c + 3]);
  }
  fmaxo[q] = sqrt(fm);
  if (mode[q] != TM_SERVE_OPT) return;
  double dt = f[2 * q], alpha = f[2 * q + 1];
  double cv = 1.0 - alpha, cf = ff > 0 ? alpha * sqrt(vv / ff) : 0.0;
  if (fv > 0) {
    if (np[q] > kFireNmin) {
      dt = fmin(dt * 1.1, dtmax);
      alpha *= 0.99;
    }
    np[q] += 1;
  } else if (fv < 0) {
    dt *= 0.5;
    alpha = kFireAlpha0;
    np[q] = 0;
    cv = 0.0;
    cf = 0.0;
  }
  f[2 * q] = dt;
  f[2 * q + 1] = alpha;
  coef[3 * q] = cv;
  coef[3 * q + 1] = cf;
  coef[3 * q + 2] = dt;
}

// v <- cv v + cf F, then v += dt F / m (the next pre-step moves x by dt v)
__global__ void k_fire_atoms(double* __restrict__ v, const double* __restrict__ F,
                             const double* __restrict__ m, const int32_t* __restrict__ mol,
                             const int32_t* __restrict__ mode, const double* __restrict__ coef,
                             int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int q = mol[i];
  if (mode[q] != TM_SERVE_OPT) return;
  const double cv = coef[3 * q], cf = coef[3 * q + 1], dt = coef[3 * q + 2];
  for (int d = 0; d < 3; ++d) {
    const double fd = F[3 * i + d];
    v[3 * i + d] = cv * v[3 * i + d] + cf * fd + dt * 1e-10 * fd / m[i];
  }
}

// x += dt v for the atoms of optimisation requests (dt of the molecule)
__global__ void k_fire_move(double* __restrict__ x, const double* __restrict__ v,
                            const int32_t* __restrict__ mol, const int32_t* __restrict__ mode,
                            const double* __restrict__ f, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int q = mol[i];
  if (mode[q] != TM_SERVE_OPT) return;
  const double dt = f[2 * q];
  double st[3], n2 = 0.0;
  for (int d = 0; d < 3; ++d) {
    st[d] = dt * v[3 * i + d];
    n2 += st[d] * st[d];
  }
  // no atom moves more than kFireMaxMove per step (the usual FIRE safeguard)
  const double c = !isfinite(n2) ? 0.0
                   : (n2 > kFireMaxMove * kFireMaxMove ? kFireMaxMove / sqrt(n2) : 1.0);
  if (c == 0.0) return;   // a non-finite step leaves the atom where it is
  for (int d = 0; d < 3; ++d) x[3 * i + d] += c * st[d];
}

}  // namespace

extern "C" int tm_serve_create(tm_model* model, int max_atoms, int max_mols, double dt_fs,
                               tm_serve** out) {
  if (!out) return TM_E_ARG;
  *out = nullptr;
  if (!model || max_atoms <= 0 || max_mols <= 0 || !(dt_fs > 0)) return TM_E_ARG;
  tm_ctx* ctx = model->ctx;
  tm_serve* sv = new tm_serve();
  sv->ctx = ctx;
  sv->dt = dt_fs;
  const size_t before = ctx->in_use;
  int rc = tm_system_create_capacity(model, max_atoms, max_mols, &sv->s);
  const size_t n3 = (size_t)3 * max_atoms * sizeof(double);
  if (!rc) {
    void** bufs[] = {(void**)&sv->v, (void**)&sv->a, (void**)&sv->x2, (void**)&sv->v2,
                     (void**)&sv->a2, (void**)&sv->xnew, (void**)&sv->vnew};
    for (void** b : bufs)
      if (!rc) rc = tm_alloc(ctx, b, n3);
    if (!rc) rc = tm_alloc(ctx, (void**)&sv->m, sizeof(double) * max_atoms);
    if (!rc) rc = tm_alloc(ctx, (void**)&sv->src, sizeof(int32_t) * max_atoms);
    if (!rc) rc = tm_alloc(ctx, (void**)&sv->mode, sizeof(int32_t) * max_mols);
    if (!rc) rc = tm_alloc(ctx, (void**)&sv->fire, sizeof(double) * 2 * max_mols);
    if (!rc) rc = tm_alloc(ctx, (void**)&sv->fire2, sizeof(double) * 2 * max_mols);
    if (!rc) rc = tm_alloc(ctx, (void**)&sv->npos, sizeof(int32_t) * max_mols);
    if (!rc) rc = tm_alloc(ctx, (void**)&sv->npos2, sizeof(int32_t) * max_mols);
    if (!rc) rc = tm_alloc(ctx, (void**)&sv->msrc, sizeof(int32_t) * max_mols);
    if (!rc) rc = tm_alloc(ctx, (void**)&sv->fmax, sizeof(double) * max_mols);
    if (!rc) rc = tm_alloc(ctx, (void**)&sv->coef, sizeof(double) * 3 * max_mols);
  }
  if (!rc) rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "serve create");
  sv->bytes = ctx->in_use - before;
  if (rc) {
    tm_serve_destroy(sv);
    return rc;
  }
  *out = sv;
  return TM_OK;
}

extern "C" int tm_serve_destroy(tm_serve* sv) {
  if (!sv) return TM_OK;
  tm_ctx* ctx = sv->ctx;
  const size_t cap = sv->s ? (size_t)sv->s->N_cap : 0;
  const size_t n3 = 3 * cap * sizeof(double);
  tm_free(ctx, sv->v, n3);
  tm_free(ctx, sv->a, n3);
  tm_free(ctx, sv->x2, n3);
  tm_free(ctx, sv->v2, n3);
  tm_free(ctx, sv->a2, n3);
  tm_free(ctx, sv->xnew, n3);
  tm_free(ctx, sv->vnew, n3);
  tm_free(ctx, sv->m, cap * sizeof(double));
  tm_free(ctx, sv->src, cap * sizeof(int32_t));
  const size_t mc = sv->s ? (size_t)sv->s->nmol_cap : 0;
  tm_free(ctx, sv->mode, mc * sizeof(int32_t));
  tm_free(ctx, sv->fire, mc * 2 * sizeof(double));
  tm_free(ctx, sv->fire2, mc * 2 * sizeof(double));
  tm_free(ctx, sv->npos, mc * sizeof(int32_t));
  tm_free(ctx, sv->npos2, mc * sizeof(int32_t));
  tm_free(ctx, sv->msrc, mc * sizeof(int32_t));
  tm_free(ctx, sv->fmax, mc * sizeof(double));
  tm_free(ctx, sv->coef, mc * 3 * sizeof(double));
  if (sv->s) tm_system_destroy(sv->s);
  cudaStreamSynchronize(ctx->stream);
  delete sv;
  return TM_OK;
}

extern "C" int tm_serve_info(const tm_serve* sv, int* max_atoms, int* max_mols, int* natoms,
                             int* nmol, size_t* bytes) {
  if (!sv) return TM_E_ARG;
  if (max_atoms) *max_atoms = sv->s->N_cap;
  if (max_mols) *max_mols = sv->s->nmol_cap;
  if (natoms) *natoms = sv->s->N;
  if (nmol) *nmol = sv->s->nmol;
  if (bytes) *bytes = sv->bytes;
  return TM_OK;
}

extern "C" int tm_serve_layout(tm_serve* sv, int nmol, const int32_t* Z, const int64_t* offsets,
                               const int32_t* mode, const int32_t* src, const double* x_new,
                               const double* v_new) {
  if (!sv || nmol < 0 || (nmol > 0 && (!Z || !offsets || !mode || !src))) return TM_E_ARG;
  tm_system* s = sv->s;
  tm_ctx* ctx = sv->ctx;
  if (nmol == 0) {
    s->N = 0;
    s->nmol = 0;
    return TM_OK;
  }
  const int N = (int)offsets[nmol];
  if (N > s->N_cap || nmol > s->nmol_cap) return tm_fail(ctx, TM_E_CAPACITY, "batch exceeds the serving capacity");
  int nnew = 0;
  const int Nold = s->N;
  for (int i = 0; i < N; ++i) {
    if (src[i] >= Nold) return tm_fail(ctx, TM_E_ARG, "src index beyond the previous layout");
    if (src[i] < 0) {
      if (src[i] != -(nnew + 1)) return tm_fail(ctx, TM_E_ARG, "new rows must be numbered -1, -2, ... in order");
      ++nnew;
    }
  }
  if (nnew && (!x_new || !v_new)) return TM_E_ARG;
  for (int q = 0; q < nmol; ++q)
    if (mode[q] != TM_SERVE_EF && mode[q] != TM_SERVE_MD && mode[q] != TM_SERVE_OPT)
      return tm_fail(ctx, TM_E_ARG, "serve mode");
  // previous molecule of each new molecule (from its first atom), for the
  // per-molecule optimiser state
  std::vector<int32_t> msrc(nmol, -1);
  for (int q = 0; q < nmol; ++q) {
    const int first = src[offsets[q]];
    if (first >= 0 && s->nmol > 0) {
      // the old molecule whose rows contain `first` (offsets are increasing)
      const auto it = std::upper_bound(s->off.begin(), s->off.begin() + s->nmol + 1, (int64_t)first);
      const int o = (int)(it - s->off.begin()) - 1;
      if (o >= 0 && o < s->nmol) msrc[q] = o;
    }
  }
  cudaStream_t st = ctx->stream;
  int rc;
  // upload the gather map and new rows before the layout changes the sizes
  if ((rc = tm_cuda_check(ctx, cudaMemcpyAsync(sv->src, src, sizeof(int32_t) * N, cudaMemcpyHostToDevice, st), "src")))
    return rc;
  if (nnew) {
    cudaMemcpyAsync(sv->xnew, x_new, sizeof(double) * 3 * nnew, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(sv->vnew, v_new, sizeof(double) * 3 * nnew, cudaMemcpyHostToDevice, st);
  }
  cudaMemcpyAsync(sv->mode, mode, sizeof(int32_t) * nmol, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(sv->msrc, msrc.data(), sizeof(int32_t) * nmol, cudaMemcpyHostToDevice, st);
  k_fire_gather<<<tm_div_up(nmol, 128), 128, 0, st>>>(sv->msrc, nmol, sv->fire, sv->npos, sv->fire2,
                                                      sv->npos2, sv->dt);
  ctx->launches++;
  std::swap(sv->fire, sv->fire2);
  std::swap(sv->npos, sv->npos2);
  if ((rc = tm_system_relayout(s, N, nmol, Z, offsets))) return rc;   // uploads Z, syncs
  k_serve_gather<<<tm_div_up(N, 256), 256, 0, st>>>(sv->src, N, s->d_x, sv->v, sv->a, sv->xnew,
                                                    sv->vnew, s->d_Z, sv->x2, sv->v2, sv->a2, sv->m);
  ctx->launches++;
  std::swap(s->d_x, sv->x2);
  std::swap(sv->v, sv->v2);
  std::swap(sv->a, sv->a2);
  // device errors of the gathers surface at the next step's status check
  return tm_cuda_check(ctx, cudaGetLastError(), "serve layout");
}

extern "C" int tm_serve_step(tm_serve* sv, double* E_out, double* fmax_out) {
  if (!sv) return TM_E_ARG;
  tm_system* s = sv->s;
  tm_ctx* ctx = sv->ctx;
  if (s->N == 0) return TM_OK;
  cudaStream_t st = ctx->stream;
  const int N = s->N, gb = tm_div_up(N, 256);
  k_serve_pre<<<gb, 256, 0, st>>>(s->d_x, sv->v, sv->a, s->d_mol, sv->mode, sv->dt, N);
  k_fire_move<<<gb, 256, 0, st>>>(s->d_x, sv->v, s->d_mol, sv->mode, sv->fire, N);
  ctx->launches += 2;
  int rc;
  for (int attempt = 0; attempt < 4; ++attempt) {
    if ((rc = tm_energy_force_device(s, 0))) return rc;
    bool grew = false;
    if ((rc = tm_nlist_grow(s, &grew))) return rc;   // synchronises the stream
    if (!grew) break;
    if (attempt == 3) return tm_fail(ctx, TM_E_CAPACITY, "neighbour rows keep overflowing");
  }
  k_serve_post<<<gb, 256, 0, st>>>(sv->v, sv->a, s->d_F, sv->m, s->d_mol, sv->mode, sv->dt, N);
  k_fire_chunk<<<s->nchunk, 256, 0, st>>>(s->d_chunk, s->d_mol, sv->mode, s->d_F, sv->v, s->d_part);
  k_fire_mol<<<tm_div_up(s->nmol, 128), 128, 0, st>>>(s->d_mol_chunk, s->d_part, sv->mode, sv->fire,
                                                      sv->npos, sv->coef, sv->fmax, s->nmol,
                                                      kFireDtMax * sv->dt);
  k_fire_atoms<<<gb, 256, 0, st>>>(sv->v, s->d_F, sv->m, s->d_mol, sv->mode, sv->coef, N);
  ctx->launches += 4;
  if (fmax_out &&
      (rc = tm_cuda_check(ctx, cudaMemcpyAsync(fmax_out, sv->fmax, sizeof(double) * s->nmol,
                                               cudaMemcpyDeviceToHost, st), "fmax")))
    return rc;
  if (E_out &&
      (rc = tm_cuda_check(ctx, cudaMemcpyAsync(E_out, s->d_mol_E, sizeof(double) * 4 * s->nmol,
                                               cudaMemcpyDeviceToHost, st), "energies")))
    return rc;
  return tm_sync_status(ctx, "serve step");
}

extern "C" int tm_serve_read(tm_serve* sv, int mol, double* x, double* v, double* F) {
  if (!sv || mol < 0 || mol >= sv->s->nmol) return TM_E_ARG;
  tm_system* s = sv->s;
  tm_ctx* ctx = sv->ctx;
  const int64_t a0 = s->off[mol], n = s->off[mol + 1] - a0;
  cudaStream_t st = ctx->stream;
  const size_t bytes = sizeof(double) * 3 * n;
  if (x) cudaMemcpyAsync(x, s->d_x + 3 * a0, bytes, cudaMemcpyDeviceToHost, st);
  if (v) cudaMemcpyAsync(v, sv->v + 3 * a0, bytes, cudaMemcpyDeviceToHost, st);
  if (F) cudaMemcpyAsync(F, s->d_F + 3 * a0, bytes, cudaMemcpyDeviceToHost, st);
  return tm_cuda_check(ctx, cudaStreamSynchronize(st), "serve read");
}
