// Network outputs -> per-atom energies/charges, charge neutralisation, the
// DSF/elu Coulomb and Grimme-C6 vdW pair terms, and the per-molecule totals.
//
// Reference: dipole_inference / energy_inference (TFNetworks/
// TFBehlerParinelloSymEE.py:884-1015), TFCoulombEluSRDSFLR (TFDescriptors/
// RawSymFunc.py:1307-1359), TFVdwPolyLR (RawSymFunc.py:1361-1414); periodic
// halving TFBehlerParinelloSymEE.py:1550, 1620.
//
// Pair terms are evaluated without a stored pair list: each warp takes up to
// eight atoms of one cell and sweeps the cells whose boxes come within the
// Coulomb cutoff, lanes striding over candidate atoms. Every pair is evaluated
// from both ends (a gather), so per-atom sums need no atomics and are
// deterministic. Membership uses the same FP32 screen + exact FP64 rule as the
// neighbour lists. Energies are returned as half-pair sums per atom and
// reduced per molecule in FP64.
#include <cuda_runtime.h>

#include "tm_internal.h"

namespace {

constexpr float kBand = 1e-5f;
constexpr int GI = 8;   // centre atoms per warp

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
                             float* __restrict__ q, int N) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int m = mol[i];
  const double n = (double)(off[m + 1] - off[m]);
  q[i] = (float)((double)qraw[i] - aux[8 * m] / n);   // TFBehlerParinelloSymEE.py:1006-1009
}

struct CoulArgs {
  const double* x;
  const float4* xhi;
  const float4* xlo;
  const float* q;
  const int32_t* mol;
  const tm_grid* grid;
  const int32_t* cell_start;
  const int32_t* cell_atoms;
  const int32_t* ncell;
  int ncell_cap;
  double* ecv;       // [N][2]
  float* dEdqt;      // [N]  dE/d q~_i
  float4* fcv;       // [N]  dE/dx_i of the pair terms
  int ref_periodic;  // image pairs contribute half the force (reference gradient)
  int periodic;
  double ree;
  float ree2_lo, ree2_hi;
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
        kc = ec / rb - k.zz + (rb - k.r_lr) * (k.zz / k.r_lr + k.yy);
        dkc = -(ec / (rb * rb) + 1.1283791671f * k.alpha * expf(-ar * ar) / rb) +
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
    const float den = 1.f + 6.f * x12;
    const float damp = 1.f / den;
    const float K = -cut * s6 * inv6 * damp;
    // d damp / d rp = 72 x12 / (rp den^2)
    const float dK = -s6 * (dcut * inv6 * damp - 6.f * cut * inv6 * inv * damp +
                            cut * inv6 * 72.f * x12 * inv * damp * damp);
    o.e_vdw = K;
    o.dedr += dK * b2;
  }
  return o;
}

__global__ void __launch_bounds__(128) k_coulomb(const CoulArgs a, const tm_consts k) {
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * (blockDim.x >> 5) + wib;
  if (c >= *a.ncell) return;
  const int t0 = a.cell_start[c], t1 = a.cell_start[c + 1];
  if (t1 <= t0) return;
  const int m = a.mol[a.cell_atoms[t0]];
  const tm_grid g = a.grid[m];
  const int lc = c - g.cell_off;
  const int iz = lc % g.nz, iy = (lc / g.nz) % g.ny, ix = lc / (g.nz * g.ny);
  const int Rx = (int)ceil(a.ree / g.cx), Ry = (int)ceil(a.ree / g.cy), Rz = (int)ceil(a.ree / g.cz);
  const double ree2 = a.ree * a.ree;
  for (int gb = t0; gb < t1; gb += GI) {
    const int ng = min(GI, t1 - gb);
    int ia[GI];
    float4 hi[GI], lo[GI];
    float qi[GI];
    int ei[GI];
    float acc_cc[GI], acc_vdw[GI], gx[GI], gy[GI], gz[GI];
#pragma unroll
    for (int u = 0; u < GI; ++u) {
      const int t = gb + (u < ng ? u : 0);
      ia[u] = a.cell_atoms[t];
      hi[u] = a.xhi[ia[u]];
      lo[u] = a.xlo[ia[u]];
      qi[u] = a.q[ia[u]];
      ei[u] = __float_as_int(hi[u].w);
      acc_cc[u] = acc_vdw[u] = gx[u] = gy[u] = gz[u] = 0.f;
    }
    for (int ox = -Rx; ox <= Rx; ++ox) {
      const double gapx = fmax(0.0, fabs((double)ox) - 1.0) * g.cx;
      for (int oy = -Ry; oy <= Ry; ++oy) {
        const double gapy = fmax(0.0, fabs((double)oy) - 1.0) * g.cy;
        for (int oz = -Rz; oz <= Rz; ++oz) {
          const double gapz = fmax(0.0, fabs((double)oz) - 1.0) * g.cz;
          // boxes of the two cells are at least this far apart
          if (gapx * gapx + gapy * gapy + gapz * gapz > ree2) continue;
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
          const float shh[3] = {a.sh_hi[r][0], a.sh_hi[r][1], a.sh_hi[r][2]};
          const float shl[3] = {a.sh_lo[r][0], a.sh_lo[r][1], a.sh_lo[r][2]};
          const float fscale = (a.ref_periodic && r != TM_IMG_SELF) ? 0.5f : 1.f;
          const int u0 = a.cell_start[cj], u1 = a.cell_start[cj + 1];
          for (int tb = u0; tb < u1; tb += 32) {
            const int t = tb + lane;
            if (t >= u1) continue;
            const int j = a.cell_atoms[t];
            const float4 hj = a.xhi[j], lj = a.xlo[j];
            const float qj = a.q[j];
            const int ej = __float_as_int(hj.w);
#pragma unroll
            for (int u = 0; u < GI; ++u) {
              if (u >= ng) continue;
              if (j == ia[u] && r == TM_IMG_SELF) continue;
              const float dx = ds_sub_shift(hi[u].x, lo[u].x, hj.x, lj.x, shh[0], shl[0]);
              const float dy = ds_sub_shift(hi[u].y, lo[u].y, hj.y, lj.y, shh[1], shl[1]);
              const float dz = ds_sub_shift(hi[u].z, lo[u].z, hj.z, lj.z, shh[2], shl[2]);
              const float d2 = dx * dx + dy * dy + dz * dz;
              if (d2 > a.ree2_hi) continue;
              if (d2 >= a.ree2_lo) {
                const int i = ia[u];
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
              const PairOut po = pair_terms(rr, qi[u], qj, ei[u], ej, k);
              acc_cc[u] += po.e_cc;
              acc_vdw[u] += po.e_vdw;
              const float s = fscale * po.dedr / rr;
              gx[u] += s * dx;
              gy[u] += s * dy;
              gz[u] += s * dz;
            }
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < GI; ++u) {
      const float c0 = warp_sum(acc_cc[u]);
      const float c1 = warp_sum(acc_vdw[u]);
      const float fx = warp_sum(gx[u]);
      const float fy = warp_sum(gy[u]);
      const float fz = warp_sum(gz[u]);
      if (lane == 0 && u < ng) {
        const int i = ia[u];
        a.ecv[2 * i + 0] = 0.5 * (double)qi[u] * (double)c0;
        a.ecv[2 * i + 1] = 0.5 * (double)c1;
        a.dEdqt[i] = c0;
        a.fcv[i] = make_float4(fx, fy, fz, 0.f);
      }
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
                                                              s->d_mol_aux, s->d_q, s->N);
  ctx->launches += 3;
  return tm_cuda_check(ctx, cudaGetLastError(), "mlp finish");
}

int tm_launch_coulomb(tm_system* s, unsigned flags) {
  tm_ctx* ctx = s->ctx;
  const tm_consts& k = s->model->k;
  CoulArgs a;
  a.x = s->d_x; a.xhi = s->d_xhi; a.xlo = s->d_xlo; a.q = s->d_q; a.mol = s->d_mol;
  a.grid = s->d_grid; a.cell_start = s->d_cell_start; a.cell_atoms = s->d_cell_atoms;
  a.ncell = s->d_ncell; a.ncell_cap = s->ncell_cap; a.ecv = s->d_ecv; a.dEdqt = s->d_dEdq;
  a.fcv = s->d_fcv;
  a.ref_periodic = (s->periodic && (flags & TM_F_REFERENCE_PERIODIC_FORCE)) ? 1 : 0;
  a.periodic = s->periodic ? 1 : 0;
  a.ree = k.ree_d;
  a.ree2_lo = (float)(k.ree_d * k.ree_d) * (1.f - kBand);
  a.ree2_hi = (float)(k.ree_d * k.ree_d) * (1.f + kBand);
  for (int q = 0; q < 9; ++q) a.lat[q] = s->lat[q];
  tm_fill_shifts(s, a.sh_hi, a.sh_lo);
  k_coulomb<<<tm_div_up(s->ncell_cap, 4), 128, 0, ctx->stream>>>(a, k);
  k_mol_sum2<<<s->nmol, 256, 0, ctx->stream>>>(s->d_off, s->d_ecv, s->d_dEdq, s->d_q, s->d_x,
                                               (double)k.bohr, s->d_mol_E, s->d_mol_aux);
  k_dq<<<tm_div_up(s->N, 256), 256, 0, ctx->stream>>>(s->d_mol, s->d_off, s->d_mol_aux, s->d_dEdq,
                                                      s->N);
  ctx->launches += 3;
  return tm_cuda_check(ctx, cudaGetLastError(), "coulomb");
}
