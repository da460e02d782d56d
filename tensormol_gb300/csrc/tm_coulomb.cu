// Network outputs -> per-atom energies/charges, charge neutralisation, the
// DSF/elu Coulomb and Grimme-C6 vdW pair terms, and the per-molecule totals.
//
// Reference: dipole_inference / energy_inference (TFNetworks/
// TFBehlerParinelloSymEE.py:884-1015), TFCoulombEluSRDSFLR (TFDescriptors/
// RawSymFunc.py:1307-1359), TFVdwPolyLR (RawSymFunc.py:1361-1414); periodic
// halving TFBehlerParinelloSymEE.py:1550, 1620.
//
// Pair terms are evaluated without a stored pair list, on a second cell grid
// sized for about 24 atoms per cell with the atoms packed in cell order: one
// warp per cell, lane = centre atom; the cells whose boxes come within the
// Coulomb cutoff are staged 32 atoms at a time in shared memory and read by
// all lanes as broadcasts. Every pair is evaluated from both ends (a gather),
// so per-atom sums need no atomics and are deterministic. Membership uses the
// same FP32 screen + exact FP64 rule as the neighbour lists. Energies are
// returned as half-pair sums per atom and reduced per molecule in FP64.
#include <cuda_runtime.h>

#include "tm_internal.h"

namespace {

constexpr float kBand = 1e-5f;

__global__ void k_mlp_finish(const float* __restrict__ epart, const double* __restrict__ bout,
                             const int32_t* __restrict__ row_of_atom,
                             const int32_t* __restrict__ elem, int nsplit, int Mpad, int nele,
                             int N, double* __restrict__ Eatom, float* __restrict__ qraw) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int row = row_of_atom[i], e = elem[i];
  double E = bout[e], q = bout[nele + e];
  for (int s = 0; s < nsplit; ++s) {
    E += (double)epart[(size_t)row * nsplit + s];
    q += (double)epart[((size_t)Mpad + row) * nsplit + s];
  }
  Eatom[i] = E;
  qraw[i] = (float)q;
}

// block per molecule: aux[m][0] = sum q_raw, mol_E[m][1] = Ebp
__global__ void k_mol_sum1(const int32_t* __restrict__ off, const double* __restrict__ Eatom,
                           const float* __restrict__ qraw, double* __restrict__ molE,
                           double* __restrict__ aux) {
  const int m = blockIdx.x;
  __shared__ double s0[256], s1[256];
  double a = 0.0, b = 0.0;
  for (int i = off[m] + threadIdx.x; i < off[m + 1]; i += blockDim.x) {
    a += Eatom[i];
    b += (double)qraw[i];
  }
  s0[threadIdx.x] = a;
  s1[threadIdx.x] = b;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s0[threadIdx.x] += s0[threadIdx.x + o];
      s1[threadIdx.x] += s1[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    molE[4 * m + 1] = s0[0];
    aux[8 * m + 0] = s1[0];
  }
}

__global__ void k_neutralize(const int32_t* __restrict__ mol, const int32_t* __restrict__ off,
                             const float* __restrict__ qraw, const double* __restrict__ aux,
                             float* __restrict__ q, const int32_t* __restrict__ epos,
                             float4* __restrict__ exlo, int N) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int m = mol[i];
  const double n = (double)(off[m + 1] - off[m]);
  const float qi = (float)((double)qraw[i] - aux[8 * m] / n);   // TFBehlerParinelloSymEE.py:1006-1009
  q[i] = qi;
  exlo[epos[i]].w = qi;
}

struct CoulArgs {
  const double* x;
  const float4* exhi;       // cell-ordered hi parts (w = element)
  const float4* exlo;       // cell-ordered lo parts (w = charge)
  const int32_t* eatom;     // cell-ordered atom index
  const int32_t* mol;
  const tm_grid* grid;      // Coulomb grid per molecule
  const int32_t* cell_start;
  const int32_t* ncell;
  int ncell_cap;
  double* ecv;              // [N][2]
  float* dEdqt;             // [N]  dE/d q~_i
  float4* fcv;              // [N]  dE/dx_i of the pair terms
  int ref_periodic;         // image pairs contribute half the force (reference gradient)
  int periodic;
  double ree;
  float ree2, ree2_lo, ree2_hi;
  double lat[9];
  float sh_hi[27][3];
  float sh_lo[27][3];
};

struct PairOut {
  float e_cc;   // q_j * k(r)           (energy = 0.5 * q_i * sum)
  float e_vdw;  // K_vdw                (energy = 0.5 * sum)
  float dedr;   // dE/dr (Angstrom) of the pair
};

__device__ __forceinline__ PairOut pair_terms(float r, float qi, float qj, int ei, int ej,
                                              const tm_consts& k) {
  PairOut o{0.f, 0.f, 0.f};
  if (k.add_ecc) {
    const float rb = r * k.bohr;
    float kc, dkc;
    if (rb > k.r_sr) {
      if (rb > k.r_lr) {
        kc = 0.f;
        dkc = 0.f;
      } else {
        const float ar = k.alpha * rb;
        const float ec = erfcf(ar);
        const float ir = 1.f / rb;
        kc = ec * ir - k.zz + (rb - k.r_lr) * (k.zz / k.r_lr + k.yy);
        dkc = -(ec * ir * ir + 1.1283791671f * k.alpha * expf(-ar * ar) * ir) +
              (k.zz / k.r_lr + k.yy);
      }
    } else {
      const float ex = expf(rb - k.r_sr);
      kc = k.elu_a * (ex - 1.f) + k.elu_shift;
      dkc = k.elu_a * ex;
    }
    o.e_cc = qj * kc;
    o.dedr = qi * qj * dkc * k.bohr;
  }
  if (k.has_vdw) {
    const float b2 = k.bohr * k.bohr;
    const float rp = r * b2;
    const float t = (rp - k.vdw_begin) / k.vdw_width;
    float cut, dcut;
    if (t > 1.f) { cut = 1.f; dcut = 0.f; }
    else if (t > 0.f) { cut = -t * t * (2.f * t - 3.f); dcut = -6.f * t * (t - 1.f) / k.vdw_width; }
    else { cut = 0.f; dcut = 0.f; }
    const float s6 = sqrtf(k.c6[ei] * k.c6[ej]);
    const float R0 = k.r0[ei] + k.r0[ej];
    const float inv = 1.f / rp;
    const float inv2 = inv * inv;
    const float inv6 = inv2 * inv2 * inv2;
    const float xr = R0 * inv;                       // (rp/R0)^-1
    const float x2 = xr * xr, x4 = x2 * x2, x12 = x4 * x4 * x4;
    const float damp = 1.f / (1.f + 6.f * x12);
    const float K = -cut * s6 * inv6 * damp;
    // d damp / d rp = 72 x12 / (rp (1 + 6 x12)^2)
    const float dK = -s6 * inv6 * damp * (dcut - 6.f * cut * inv + 72.f * cut * x12 * inv * damp);
    o.e_vdw = K;
    o.dedr += dK * b2;
  }
  return o;
}

// One warp per Coulomb-grid cell; lane = centre atom (cells with more than 32
// atoms loop). Candidate cells are culled by box distance and staged 32 atoms
// at a time in shared memory, read back as broadcasts by every lane.
__global__ void __launch_bounds__(128) k_coulomb(const CoulArgs a, const tm_consts k) {
  __shared__ float4 sh[4][2][32];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * (blockDim.x >> 5) + wib;
  if (c >= a.ncell_cap || c >= *a.ncell) return;
  const int t0 = a.cell_start[c], t1 = a.cell_start[c + 1];
  if (t1 <= t0) return;
  const tm_grid g = a.grid[a.mol[a.eatom[t0]]];
  const int lc = c - g.cell_off;
  const int iz = lc % g.nz, iy = (lc / g.nz) % g.ny, ix = lc / (g.nz * g.ny);
  const float cx = (float)g.cx, cy = (float)g.cy, cz = (float)g.cz;
  const int Rx = (int)ceil(a.ree / g.cx), Ry = (int)ceil(a.ree / g.cy), Rz = (int)ceil(a.ree / g.cz);
  float4* sj_hi = sh[wib][0];
  float4* sj_lo = sh[wib][1];
  for (int ib = t0; ib < t1; ib += 32) {
    const int ti = ib + lane;
    const bool have = ti < t1;
    const float4 hi = a.exhi[have ? ti : t0];
    const float4 lo = a.exlo[have ? ti : t0];
    const int ei = __float_as_int(hi.w);
    const float qi = lo.w;
    float acc_cc = 0.f, acc_vdw = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
    for (int ox = -Rx; ox <= Rx; ++ox) {
      const float gapx = fmaxf(0.f, (float)(abs(ox) - 1)) * cx;
      for (int oy = -Ry; oy <= Ry; ++oy) {
        const float gapy = fmaxf(0.f, (float)(abs(oy) - 1)) * cy;
        for (int oz = -Rz; oz <= Rz; ++oz) {
          const float gapz = fmaxf(0.f, (float)(abs(oz) - 1)) * cz;
          if (gapx * gapx + gapy * gapy + gapz * gapz > a.ree2_hi) continue;
          int jx = ix + ox, jy = iy + oy, jz = iz + oz, sx = 0, sy = 0, sz = 0;
          if (a.periodic) {
            if (jx < 0) { jx += g.nx; sx = -1; } else if (jx >= g.nx) { jx -= g.nx; sx = 1; }
            if (jy < 0) { jy += g.ny; sy = -1; } else if (jy >= g.ny) { jy -= g.ny; sy = 1; }
            if (jz < 0) { jz += g.nz; sz = -1; } else if (jz >= g.nz) { jz -= g.nz; sz = 1; }
          } else if (jx < 0 || jx >= g.nx || jy < 0 || jy >= g.ny || jz < 0 || jz >= g.nz) {
            continue;
          }
          const int cj = g.cell_off + (jx * g.ny + jy) * g.nz + jz;
          const int r = 9 * (sx + 1) + 3 * (sy + 1) + (sz + 1);
          const float shx = a.sh_hi[r][0], shy = a.sh_hi[r][1], shz = a.sh_hi[r][2];
          const float slx = a.sh_lo[r][0], sly = a.sh_lo[r][1], slz = a.sh_lo[r][2];
          const float fscale = (a.ref_periodic && r != TM_IMG_SELF) ? 0.5f : 1.f;
          const int u0 = a.cell_start[cj], u1 = a.cell_start[cj + 1];
          for (int jb = u0; jb < u1; jb += 32) {
            const int nj = min(32, u1 - jb);
            __syncwarp();
            if (lane < nj) {
              sj_hi[lane] = a.exhi[jb + lane];
              sj_lo[lane] = a.exlo[jb + lane];
            }
            __syncwarp();
            if (!have) continue;
            for (int q = 0; q < nj; ++q) {
              if (cj == c && jb + q == ti && r == TM_IMG_SELF) continue;   // the atom itself
              const float4 hj = sj_hi[q], lj = sj_lo[q];
              const float dx = ds_sub_shift(hi.x, lo.x, hj.x, lj.x, shx, slx);
              const float dy = ds_sub_shift(hi.y, lo.y, hj.y, lj.y, shy, sly);
              const float dz = ds_sub_shift(hi.z, lo.z, hj.z, lj.z, shz, slz);
              const float d2 = dx * dx + dy * dy + dz * dz;
              if (d2 > a.ree2_hi) continue;
              if (d2 >= a.ree2_lo) {   // within 1e-5 of the cutoff: the exact FP64 rule
                const int i = a.eatom[ti], j = a.eatom[jb + q];
                double xj = a.x[3 * j], yj = a.x[3 * j + 1], zj = a.x[3 * j + 2];
                if (a.periodic) {
                  xj = tm_image_coord(xj, sx, sy, sz, a.lat[0], a.lat[3], a.lat[6]);
                  yj = tm_image_coord(yj, sx, sy, sz, a.lat[1], a.lat[4], a.lat[7]);
                  zj = tm_image_coord(zj, sx, sy, sz, a.lat[2], a.lat[5], a.lat[8]);
                }
                if (!tm_exact_within(a.x[3 * i], a.x[3 * i + 1], a.x[3 * i + 2], xj, yj, zj, a.ree))
                  continue;
              }
              const float rr = sqrtf(d2);
              const PairOut po = pair_terms(rr, qi, lj.w, ei, __float_as_int(hj.w), k);
              acc_cc += po.e_cc;
              acc_vdw += po.e_vdw;
              const float sc = fscale * po.dedr / rr;
              gx += sc * dx;
              gy += sc * dy;
              gz += sc * dz;
            }
          }
        }
      }
    }
    if (have) {
      const int i = a.eatom[ti];
      a.ecv[2 * i + 0] = 0.5 * (double)qi * (double)acc_cc;
      a.ecv[2 * i + 1] = 0.5 * (double)acc_vdw;
      a.dEdqt[i] = acc_cc;
      a.fcv[i] = make_float4(gx, gy, gz, 0.f);
    }
  }
}

// block per molecule: Ecc, Evdw, Etotal, dipole, sum dE/dq~
__global__ void k_mol_sum2(const int32_t* __restrict__ off, const double* __restrict__ ecv,
                           const float* __restrict__ dEdqt, const float* __restrict__ q,
                           const double* __restrict__ x, double bohr, double* __restrict__ molE,
                           double* __restrict__ aux) {
  const int m = blockIdx.x;
  __shared__ double s[6][256];
  double v[6] = {0, 0, 0, 0, 0, 0};
  for (int i = off[m] + threadIdx.x; i < off[m + 1]; i += blockDim.x) {
    v[0] += ecv[2 * i];
    v[1] += ecv[2 * i + 1];
    v[2] += (double)dEdqt[i];
    const double qq = (double)q[i];
    v[3] += qq * x[3 * i] * bohr;
    v[4] += qq * x[3 * i + 1] * bohr;
    v[5] += qq * x[3 * i + 2] * bohr;
  }
  for (int c = 0; c < 6; ++c) s[c][threadIdx.x] = v[c];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int c = 0; c < 6; ++c) s[c][threadIdx.x] += s[c][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    molE[4 * m + 2] = s[0][0];
    molE[4 * m + 3] = s[1][0];
    molE[4 * m + 0] = molE[4 * m + 1] + s[0][0] + s[1][0];
    aux[8 * m + 1] = s[2][0];
    aux[8 * m + 2] = s[3][0];
    aux[8 * m + 3] = s[4][0];
    aux[8 * m + 4] = s[5][0];
  }
}

// dE/dq_i = dE/dq~_i - (1/N) sum_k dE/dq~_k (adjoint of the neutralisation)
__global__ void k_dq(const int32_t* __restrict__ mol, const int32_t* __restrict__ off,
                     const double* __restrict__ aux, float* __restrict__ dEdq, int N) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int m = mol[i];
  const double n = (double)(off[m + 1] - off[m]);
  dEdq[i] = (float)((double)dEdq[i] - aux[8 * m + 1] / n);
}

}  // namespace

void tm_fill_shifts(const tm_system* s, float hi[27][3], float lo[27][3]);

int tm_launch_mlp_finish(tm_system* s) {
  tm_ctx* ctx = s->ctx;
  tm_model* m = s->model;
  const int nsplit = m->H / TM_BN;
  k_mlp_finish<<<tm_div_up(s->N, 256), 256, 0, ctx->stream>>>(
      s->epart, m->bout, s->row_of_atom, s->d_elem, nsplit, s->Mpad, m->k.nele, s->N, s->d_Eatom,
      s->d_qraw);
  k_mol_sum1<<<s->nmol, 256, 0, ctx->stream>>>(s->d_off, s->d_Eatom, s->d_qraw, s->d_mol_E,
                                               s->d_mol_aux);
  k_neutralize<<<tm_div_up(s->N, 256), 256, 0, ctx->stream>>>(s->d_mol, s->d_off, s->d_qraw,
                                                              s->d_mol_aux, s->d_q, s->d_epos,
                                                              s->d_exlo, s->N);
  ctx->launches += 3;
  return tm_cuda_check(ctx, cudaGetLastError(), "mlp finish");
}

int tm_launch_coulomb(tm_system* s, unsigned flags) {
  tm_ctx* ctx = s->ctx;
  const tm_consts& k = s->model->k;
  CoulArgs a;
  a.x = s->d_x; a.exhi = s->d_exhi; a.exlo = s->d_exlo; a.eatom = s->d_ecell_atoms;
  a.mol = s->d_mol; a.grid = s->d_egrid; a.cell_start = s->d_ecell_start; a.ncell = s->d_encell;
  a.ncell_cap = s->ecell_cap; a.ecv = s->d_ecv; a.dEdqt = s->d_dEdq; a.fcv = s->d_fcv;
  a.ref_periodic = (s->periodic && (flags & TM_F_REFERENCE_PERIODIC_FORCE)) ? 1 : 0;
  a.periodic = s->periodic ? 1 : 0;
  a.ree = k.ree_d;
  a.ree2 = (float)(k.ree_d * k.ree_d);
  a.ree2_lo = a.ree2 * (1.f - kBand);
  a.ree2_hi = a.ree2 * (1.f + kBand);
  for (int q = 0; q < 9; ++q) a.lat[q] = s->lat[q];
  tm_fill_shifts(s, a.sh_hi, a.sh_lo);
  k_coulomb<<<tm_div_up(s->ecell_cap, 4), 128, 0, ctx->stream>>>(a, k);
  k_mol_sum2<<<s->nmol, 256, 0, ctx->stream>>>(s->d_off, s->d_ecv, s->d_dEdq, s->d_q, s->d_x,
                                               (double)k.bohr, s->d_mol_E, s->d_mol_aux);
  k_dq<<<tm_div_up(s->N, 256), 256, 0, ctx->stream>>>(s->d_mol, s->d_off, s->d_mol_aux, s->d_dEdq,
                                                      s->N);
  ctx->launches += 3;
  return tm_cuda_check(ctx, cudaGetLastError(), "coulomb");
}
