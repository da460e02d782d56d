// Network outputs -> per-atom energies/charges, charge neutralisation, the
// DSF/elu Coulomb and Grimme-C6 vdW pair terms, and the per-molecule totals.
//
// Reference: dipole_inference / energy_inference (TFNetworks/
// TFBehlerParinelloSymEE.py:884-1015), TFCoulombEluSRDSFLR (TFDescriptors/
// RawSymFunc.py:1307-1359), TFVdwPolyLR (RawSymFunc.py:1361-1414); periodic
// halving TFBehlerParinelloSymEE.py:1550, 1620.
//
// Pair terms are evaluated without a stored pair list, on a second cell grid
// sized for about 24 atoms per cell with the atoms packed in cell order. One
// warp per (centre block, share of the stencil): a centre block is a run of
// up to 32 consecutive atoms of one (x, y) column of cells, lane = centre.
// Candidates come from the upper half of the stencil (column offsets after
// (0, 0) in x-major order; in the own column, the atoms after the centre in
// cell order), so every pair is evaluated once (Newton's third law). They are
// staged in shared memory after a screen against the centres' bounding box
// and taken by all lanes in the same order. The centre's sums stay in
// registers; the reaction on a candidate (its dE/dq~ share and gradient) is
// summed over the lanes by a butterfly and added into per-atom 64-bit
// fixed-point totals in global memory. Integer addition is associative, so
// the totals are bit-identical whatever order the warps add them in. The vdW
// energy of a pair is booked whole at the centre. Membership uses the same
// FP32 screen + exact FP64 rule as the neighbour lists. Per-molecule energies
// are reduced in FP64.
#include <cuda_runtime.h>

#include <climits>

#include "tm_internal.h"

namespace {

constexpr float kBand = 1e-5f;

// Per-molecule sums in two fixed-order levels: one block per chunk of at most
// TM_CHUNK atoms of one molecule, then one warp per molecule over its chunks.
template <int NV>
__device__ __forceinline__ void block_sum_store(double (&v)[NV], double* __restrict__ dst) {
  __shared__ double sh[NV][256];
  for (int c = 0; c < NV; ++c) sh[c][threadIdx.x] = v[c];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int c = 0; c < NV; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < NV; ++c) dst[c] = sh[c][0];
}

// Network outputs -> per-atom energy and raw charge (output bias plus the
// N-tile partials of the last layer), and the chunk partials [c][0] = sum
// Eatom, [c][1] = sum q_raw: one block per chunk.
__global__ void k_mlp_finish(const int2* __restrict__ chunk, const float* __restrict__ epart,
                             const double* __restrict__ bout, const int32_t* __restrict__ row_of_atom,
                             const int32_t* __restrict__ elem, int nsplit, int Mpad, int nele,
                             double* __restrict__ Eatom, float* __restrict__ qraw,
                             double* __restrict__ part) {
  const int2 ch = chunk[blockIdx.x];
  double v[2] = {0.0, 0.0};
  for (int i = ch.x + threadIdx.x; i < ch.y; i += blockDim.x) {
    const int row = row_of_atom[i], e = elem[i];
    double E = bout[e], q = bout[nele + e];
    for (int s = 0; s < nsplit; ++s) {
      E += (double)epart[(size_t)row * nsplit + s];
      q += (double)epart[((size_t)Mpad + row) * nsplit + s];
    }
    Eatom[i] = E;
    const float qf = (float)q;
    qraw[i] = qf;
    v[0] += E;
    v[1] += (double)qf;
  }
  block_sum_store<2>(v, part + 8 * (size_t)blockIdx.x);
}

// One warp per molecule: lane l adds chunks l, l + 32, ...; the lanes are then
// combined by a fixed xor butterfly (same order every call).
template <int NV>
__device__ __forceinline__ void warp_chunk_sum(const int32_t* __restrict__ mol_chunk,
                                               const double* __restrict__ part, int m, int lane,
                                               const int (&slot)[NV], double (&v)[NV]) {
  for (int t = 0; t < NV; ++t) v[t] = 0.0;
  for (int c = mol_chunk[m] + lane; c < mol_chunk[m + 1]; c += 32)
    for (int t = 0; t < NV; ++t) v[t] += part[8 * (size_t)c + slot[t]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    for (int t = 0; t < NV; ++t) v[t] += __shfl_xor_sync(TM_FULL, v[t], o);
}

__global__ void k_mol_final1(const int32_t* __restrict__ mol_chunk, const double* __restrict__ part,
                             double* __restrict__ molE, double* __restrict__ aux, int nmol) {
  const int m = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (m >= nmol) return;
  const int slot[2] = {0, 1};
  double v[2];
  warp_chunk_sum<2>(mol_chunk, part, m, lane, slot, v);
  if (lane == 0) {
    molE[4 * m + 1] = v[0];
    aux[8 * m + 0] = v[1];
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
  const float4* exhi;       // cell order: position relative to the atom's cell origin (w = element)
  const float4* exlo;       // cell order: w = charge
  const int32_t* eatom;     // cell-ordered atom index
  const int32_t* mol;
  const tm_grid* grid;      // Coulomb grid per molecule
  const int32_t* cell_start;
  const int32_t* cell_of;   // [N] Coulomb cell of each atom
  const int4* blk;          // centre blocks (column head cell, first atom, end atom)
  const int32_t* nblk;
  int blk_cap;
  double* ecv;              // [N][2]
  float* dEdqt;             // [N]  dE/d q~_i
  float4* fcv;              // [N]  dE/dx_i of the pair terms
  unsigned long long* acc;  // [5][N] fixed-point sums (cell order): cc, vdw, dE/dx xyz
  tm_dev_status* st;
  int natoms;
  int ref_periodic;         // image pairs contribute half the force (reference gradient)
  int periodic;
  double ree;
  float ree2, ree2_lo, ree2_hi;
  double reach;             // cell search radius: cutoff + skin (cells from an earlier build)
  float reach2;
  float pre2;               // candidate-vs-centre-box screen: ree^2 (1 + 2e-5)
  float inv_bohr, inv_b2, inv_vdw_width, c_lin;   // 1/bohr, 1/bohr^2, 1/width, zz/R_lr + yy
  double lat[9];
  int ortho;                // periodic: orthorhombic cell
  double cu[9];             // periodic, not orthorhombic: grid-cell edges a_d / n_d (rows)
  float sh_hi[27][3];
  float sh_lo[27][3];
};

struct PairOut {
  float kc;     // k(r): the centre's sum takes q_j * k, the candidate's q_i * k
  float e_vdw;  // K_vdw                (the pair's energy, booked at the centre)
  float dedr;   // dE/dr (Angstrom) of the pair
};

// 2^32 fixed-point units per Hartree (per Hartree/A for the gradient):
// resolution 2.3e-10, range +-2.1e9.
constexpr float kFixScale = 4294967296.f;
constexpr double kFixInv = 1.0 / 4294967296.0;

// Adds v to a 2^-32 fixed-point total in global memory; |v| >= 2^31 (only
// non-finite or absurd charges reach it) flags the status word instead.
__device__ __forceinline__ void add_fix(unsigned long long* dst, float v, tm_dev_status* st) {
  if (!(fabsf(v) < 2.0e9f)) {
    tm_flag(st, TM_E_NONFINITE, 0, 3);
    return;
  }
  const long long t = __float2ll_rn(v * kFixScale);
  if (t) atomicAdd(dst, (unsigned long long)t);
}

// r in Angstrom and ir = 1/r; s6 = sqrt(C6_i C6_j), R0 = R0_i + R0_j of the pair.
__device__ __forceinline__ PairOut pair_terms(float r, float ir, float qi, float qj, float s6,
                                              float R0, const CoulArgs& a, const tm_consts& k) {
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
        // exp(-x^2) with the rounding error of x^2 (exact by an FMA) folded in
        const float x2 = ar * ar;
        const float ex2 = expf(-x2) * (1.f - fmaf(ar, ar, -x2));
        float ec;
        if (k.erfc_n) {   // exp(-x^2) erfcx(x), erfcx by its polynomial on this range
          const float t = fmaf(ar, k.erfc_s, k.erfc_o);
          float pp = k.erfc_c[10];
#pragma unroll
          for (int e = 9; e >= 0; --e) pp = fmaf(pp, t, k.erfc_c[e]);
          ec = ex2 * pp;
        } else {
          ec = erfcf(ar);
        }
        const float irb = ir * a.inv_bohr;
        kc = ec * irb - k.zz + (rb - k.r_lr) * a.c_lin;
        dkc = a.c_lin - irb * (ec * irb + 1.1283791671f * k.alpha * ex2);
      }
    } else {
      const float ex = expf(rb - k.r_sr);
      kc = k.elu_a * (ex - 1.f) + k.elu_shift;
      dkc = k.elu_a * ex;
    }
    o.kc = kc;
    o.dedr = qi * qj * dkc * k.bohr;
  }
  if (k.has_vdw) {
    const float b2 = k.bohr * k.bohr;
    const float rp = r * b2;
    const float t = (rp - k.vdw_begin) * a.inv_vdw_width;
    float cut, dcut;
    if (t > 1.f) { cut = 1.f; dcut = 0.f; }
    else if (t > 0.f) { cut = -t * t * (2.f * t - 3.f); dcut = -6.f * t * (t - 1.f) * a.inv_vdw_width; }
    else { cut = 0.f; dcut = 0.f; }
    const float inv = ir * a.inv_b2;                  // 1 / rp
    const float inv2 = inv * inv;
    const float inv6 = inv2 * inv2 * inv2;
    const float xr = R0 * inv;                        // (rp/R0)^-1
    const float x2 = xr * xr, x4 = x2 * x2, x12 = x4 * x4 * x4;
    const float damp = __fdividef(1.f, 1.f + 6.f * x12);
    // x12 * damp = (1 - damp) / 6: finite even where x12 overflows at contact
    const float xdamp = (1.f - damp) * (1.f / 6.f);
    const float K = -cut * s6 * inv6 * damp;
    // d damp / d rp = 72 x12 / (rp (1 + 6 x12)^2)
    const float dK = -s6 * inv6 * damp * (dcut - 6.f * cut * inv + 72.f * cut * xdamp * inv);
    o.e_vdw = K;
    o.dedr += dK * b2;
  }
  return o;
}

// Positions are stored relative to the origin of each atom's cell; the
// block's centres and its staged candidates are moved into the frame of the
// block's first cell once (stencil offset x cell edge, periodic images
// included), so a pair vector is one FP32 subtraction per axis, accurate to
// about 1e-6 A. Candidate cells are culled by box distance; of their atoms,
// those within the cutoff of the centres' bounding box are staged (compacted
// by ballot, up to kStage at a time across columns) in shared memory.
constexpr int kStage = 64;

struct StageSmem {
  float4 p[kStage];                  // candidate position in the block frame (w = element)
  float q[kStage];                   // candidate charge
  uint32_t meta[kStage];             // image code << 27 | cell-order index
  int key[kStage];                   // own column: cell-order index (+ column size past a z wrap);
                                     // other columns: INT_MAX (every centre takes the pair)
  float js[4][kStage];               // reaction sums on the candidates: dE/dq~, dE/dx xyz
};

// All lanes take the staged candidates in the same order (a warp-uniform
// loop, so the broadcasts and the pair arithmetic of consecutive candidates
// overlap); a lane's centre takes candidate q if it is within the cutoff and
// the key rule allows it. The reaction on q (its dE/dq~ share and gradient)
// is summed over the lanes by an xor butterfly, which gives every lane the
// same bits, and stored once per stage.
__device__ __forceinline__ void coulomb_flush(const CoulArgs& a, const tm_consts& k,
                                              StageSmem& st, int n, int ti, bool have, float4 pi,
                                              float qi, const float* s6row, const float* r0row,
                                              float& acc_cc, float& acc_vdw, float& gx, float& gy,
                                              float& gz, int lane) {
  for (int q = 0; q < n; ++q) {
    const float4 pj = st.p[q];
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const float d2 = dx * dx + dy * dy + dz * dz;
    bool hit = have && d2 <= a.ree2_hi && st.key[q] > ti;
    const uint32_t meta = st.meta[q];
    const int r = (int)(meta >> 27);
    if (hit && d2 >= a.ree2_lo) {   // within 1e-5 of the cutoff: the exact FP64 rule
      const int jp = (int)(meta & ((1u << 27) - 1));
      const int i = a.eatom[ti], j = a.eatom[jp];
      double xj = a.x[3 * j], yj = a.x[3 * j + 1], zj = a.x[3 * j + 2];
      if (a.periodic) {
        int sx, sy, sz;
        tm_img_ijk(r, sx, sy, sz);
        xj = tm_image_coord(xj, sx, sy, sz, a.lat[0], a.lat[3], a.lat[6]);
        yj = tm_image_coord(yj, sx, sy, sz, a.lat[1], a.lat[4], a.lat[7]);
        zj = tm_image_coord(zj, sx, sy, sz, a.lat[2], a.lat[5], a.lat[8]);
      }
      hit = tm_exact_within(a.x[3 * i], a.x[3 * i + 1], a.x[3 * i + 2], xj, yj, zj, a.ree);
    }
    if (!__any_sync(TM_FULL, hit)) continue;
    float jc = 0.f, jx = 0.f, jy = 0.f, jz = 0.f;
    if (hit) {
      const float ir = rsqrtf(d2);
      const int ej = __float_as_int(pj.w);
      const float qj = st.q[q];
      const PairOut po = pair_terms(d2 * ir, ir, qi, qj, s6row[ej], r0row[ej], a, k);
      acc_cc += qj * po.kc;
      acc_vdw += po.e_vdw;
      const float fscale = (a.ref_periodic && r != TM_IMG_SELF) ? 0.5f : 1.f;
      const float sc = fscale * po.dedr * ir;
      gx += sc * dx;
      gy += sc * dy;
      gz += sc * dz;
      jc = qi * po.kc;
      jx = -sc * dx;
      jy = -sc * dy;
      jz = -sc * dz;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      jc += __shfl_xor_sync(TM_FULL, jc, o);
      jx += __shfl_xor_sync(TM_FULL, jx, o);
      jy += __shfl_xor_sync(TM_FULL, jy, o);
      jz += __shfl_xor_sync(TM_FULL, jz, o);
    }
    if (lane == (q & 31)) {
      st.js[0][q] = jc;
      st.js[1][q] = jx;
      st.js[2][q] = jy;
      st.js[3][q] = jz;
    }
  }
}

// Adds the staged candidates' reaction sums into their atoms' totals.
__device__ __forceinline__ void coulomb_drain(const CoulArgs& a, const StageSmem& st, int n,
                                              int lane) {
  for (int t = lane; t < n; t += 32) {
    const int jp = (int)(st.meta[t] & ((1u << 27) - 1));
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float v = st.js[c][t];
      if (v != 0.f) add_fix(a.acc + (size_t)(c == 0 ? 0 : c + 1) * a.natoms + jp, v, a.st);
    }
  }
}

// TRIC: a periodic cell that is not orthorhombic (grid cells are slices
// between lattice planes, spanned by the edges a_d / n_d in a.cu; a cell
// offset (ox, oy, oz) moves by ox u0 + oy u1 + oz u2, and the gaps along the
// three plane normals bound the distance by their maximum).
template <bool TRIC>
__global__ void __launch_bounds__(128, 6) k_coulomb(const CoulArgs a, const tm_consts k) {
  __shared__ StageSmem stage[4];
  __shared__ float tab[2][TM_MAX_ELE * TM_MAX_ELE];   // sqrt(C6_i C6_j), R0_i + R0_j
  {
    // the grid is sized for the block capacity: a CTA whose four centre
    // blocks all lie beyond the ones that exist leaves at once (the same
    // decision in every thread, before the barrier)
    const int nb = *a.nblk;
    bool work = false;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
      work |= (blockIdx.x * (blockDim.x >> 5) + w) % a.blk_cap < nb;
    if (!work) return;
  }
  if (threadIdx.x < k.nele * k.nele) {
    const int ei = threadIdx.x / k.nele, ej = threadIdx.x % k.nele;
    tab[0][threadIdx.x] = sqrtf(k.c6[ei] * k.c6[ej]);
    tab[1][threadIdx.x] = k.r0[ei] + k.r0[ej];
  }
  __syncthreads();
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wg = blockIdx.x * (blockDim.x >> 5) + wib;
  // split-major: the warps of a CTA share a stencil share (similar work) and
  // take neighbouring centre blocks
  const int split = wg / a.blk_cap, b = wg % a.blk_cap;
  if (b >= a.blk_cap || b >= *a.nblk) return;
  const int4 bk = a.blk[b];
  const int head = bk.x, t0 = bk.y, t1 = bk.z;
  const tm_grid g = a.grid[a.mol[a.eatom[t0]]];
  const int lc = head - g.cell_off;
  const int iy = (lc / g.nz) % g.ny, ix = lc / (g.nz * g.ny);
  // periodic: at most one wrap per axis (R <= n; edges are >= 2 * cutoff)
  const int Rx = a.periodic ? min((int)ceil(a.reach / g.cx), g.nx) : (int)ceil(a.reach / g.cx);
  const int Ry = a.periodic ? min((int)ceil(a.reach / g.cy), g.ny) : (int)ceil(a.reach / g.cy);
  const int Rz = a.periodic ? min((int)ceil(a.reach / g.cz), g.nz) : (int)ceil(a.reach / g.cz);
  if (!a.periodic) {
    // a small molecule's grid has few columns: most stencil shares lie
    // outside it, and the warp leaves before loading any centre
    const int ny2s = 2 * Ry + 1, col0s = Rx * ny2s + Ry, nhalfs = (2 * Rx + 1) * ny2s - col0s;
    bool any = false;
    for (int col = split; col < nhalfs && !any; col += TM_EE_SPLIT) {
      const int cf = col0s + col;
      const int jx = ix + cf / ny2s - Rx, jy = iy + cf % ny2s - Ry;
      any = jx >= 0 && jx < g.nx && jy >= 0 && jy < g.ny;
    }
    if (!any) return;
  }
  const int ncolumn = a.cell_start[head + g.nz] - a.cell_start[head];
  // z range of the block's cells; positions are taken in the frame of cell
  // (ix, iy, z0)
  const int z0 = (a.cell_of[a.eatom[t0]] - head), z1 = (a.cell_of[a.eatom[t1 - 1]] - head);
  const float cx = (float)g.cx, cy = (float)g.cy, cz = (float)g.cz;
  StageSmem& st = stage[wib];
  // Upper half of the (ox, oy) columns: (0, 0) first, then the columns
  // after it in x-major order (every z). In the own column, cells from z0 up
  // are staged and a centre takes a candidate only if the candidate's key
  // (cell-order index, plus the column's atom count past a periodic wrap) is
  // above its own index; the box-distance cull is symmetric in the offset, so
  // every pair (and every periodic image of it) is met exactly once.
  const int ny2 = 2 * Ry + 1;
  const int col0 = Rx * ny2 + Ry;
  const int nhalf = (2 * Rx + 1) * ny2 - col0;
  {
    const int ti = t0 + lane;
    const bool have = ti < t1;
    float4 pi = a.exhi[have ? ti : t0];
    if (have) {
      const int dzc = a.cell_of[a.eatom[ti]] - head - z0;
      if constexpr (TRIC) {
        pi.x += (float)(dzc * a.cu[6]);
        pi.y += (float)(dzc * a.cu[7]);
        pi.z += (float)(dzc * a.cu[8]);
      } else {
        pi.z += (float)(dzc * g.cz);
      }
    }
    const float qi = a.exlo[have ? ti : t0].w;
    const int ei = __float_as_int(pi.w);
    const float* s6row = tab[0] + ei * k.nele;
    const float* r0row = tab[1] + ei * k.nele;
    // bounding box of the block's centres (the lanes without one repeat t0)
    float bx0 = pi.x, by0 = pi.y, bz0 = pi.z, bx1 = pi.x, by1 = pi.y, bz1 = pi.z;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      bx0 = fminf(bx0, __shfl_xor_sync(TM_FULL, bx0, o));
      by0 = fminf(by0, __shfl_xor_sync(TM_FULL, by0, o));
      bz0 = fminf(bz0, __shfl_xor_sync(TM_FULL, bz0, o));
      bx1 = fmaxf(bx1, __shfl_xor_sync(TM_FULL, bx1, o));
      by1 = fmaxf(by1, __shfl_xor_sync(TM_FULL, by1, o));
      bz1 = fmaxf(bz1, __shfl_xor_sync(TM_FULL, bz1, o));
    }
    float acc_cc = 0.f, acc_vdw = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
    int n = 0;   // staged candidates (the stage spans columns: positions are in the block frame)
    for (int col = split; col < nhalf; col += TM_EE_SPLIT) {
      const int cf = col0 + col;
      const int ox = cf / ny2 - Rx, oy = cf % ny2 - Ry;
      const float gapx = fmaxf(0.f, (float)(abs(ox) - 1)) * cx;
      const float gapy = fmaxf(0.f, (float)(abs(oy) - 1)) * cy;
      const float offx = (float)(ox * g.cx), offy = (float)(oy * g.cy);
      for (int zc = (col == 0 ? z0 : z0 - Rz); zc <= z1 + Rz; ++zc) {
        const float gapz = fmaxf(0.f, (float)(max(z0 - zc, zc - z1) - 1)) * cz;
        if (TRIC ? fmaxf(gapx * gapx, fmaxf(gapy * gapy, gapz * gapz)) > a.reach2
                 : gapx * gapx + gapy * gapy + gapz * gapz > a.reach2)
          continue;
        int jx = ix + ox, jy = iy + oy, jz = zc, sx = 0, sy = 0, sz = 0;
        if (a.periodic) {
          if (jx < 0) { jx += g.nx; sx = -1; } else if (jx >= g.nx) { jx -= g.nx; sx = 1; }
          if (jy < 0) { jy += g.ny; sy = -1; } else if (jy >= g.ny) { jy -= g.ny; sy = 1; }
          if (jz < 0) { jz += g.nz; sz = -1; } else if (jz >= g.nz) { jz -= g.nz; sz = 1; }
        } else if (jx < 0 || jx >= g.nx || jy < 0 || jy >= g.ny || jz < 0 || jz >= g.nz) {
          continue;
        }
        const int cj = g.cell_off + (jx * g.ny + jy) * g.nz + jz;
        const uint32_t rcode = (uint32_t)(9 * (sx + 1) + 3 * (sy + 1) + (sz + 1)) << 27;
        float3 off;
        if constexpr (TRIC) {
          off.x = (float)(ox * a.cu[0] + oy * a.cu[3] + (zc - z0) * a.cu[6]);
          off.y = (float)(ox * a.cu[1] + oy * a.cu[4] + (zc - z0) * a.cu[7]);
          off.z = (float)(ox * a.cu[2] + oy * a.cu[5] + (zc - z0) * a.cu[8]);
        } else {
          off = make_float3(offx, offy, (float)((zc - z0) * g.cz));
        }
        const int kadd = col == 0 ? (sz > 0 ? ncolumn : 0) : -1;
        const int u1 = a.cell_start[cj + 1];
        for (int u0 = a.cell_start[cj]; u0 < u1; u0 += 32) {
          // one candidate per lane; kept if it comes within the cutoff of the
          // centres' box (a bound on its distance to every centre)
          const int t = u0 + lane;
          bool keep = false;
          float4 pj = make_float4(0.f, 0.f, 0.f, 0.f);
          float qj = 0.f;
          if (t < u1) {
            const float4 pr = a.exhi[t];
            pj = make_float4(pr.x + off.x, pr.y + off.y, pr.z + off.z, pr.w);
            qj = a.exlo[t].w;
            const float ex = fmaxf(0.f, fmaxf(bx0 - pj.x, pj.x - bx1));
            const float ey = fmaxf(0.f, fmaxf(by0 - pj.y, pj.y - by1));
            const float ez = fmaxf(0.f, fmaxf(bz0 - pj.z, pj.z - bz1));
            keep = ex * ex + ey * ey + ez * ez <= a.pre2;
          }
          const unsigned m = __ballot_sync(TM_FULL, keep);
          const int nk = __popc(m);
          if (n + nk > kStage) {
            __syncwarp();
            coulomb_flush(a, k, st, n, ti, have, pi, qi, s6row, r0row, acc_cc, acc_vdw, gx, gy, gz, lane);
            __syncwarp();
            coulomb_drain(a, st, n, lane);
            __syncwarp();
            n = 0;
          }
          if (keep) {
            const int pos = n + __popc(m & ((1u << lane) - 1u));
            st.p[pos] = pj;
            st.q[pos] = qj;
            st.meta[pos] = rcode | (uint32_t)t;
            st.key[pos] = kadd < 0 ? INT_MAX : t + kadd;
#pragma unroll
            for (int e = 0; e < 4; ++e) st.js[e][pos] = 0.f;
          }
          n += nk;
        }
      }
    }
    if (n) {
      __syncwarp();
      coulomb_flush(a, k, st, n, ti, have, pi, qi, s6row, r0row, acc_cc, acc_vdw, gx, gy, gz, lane);
      __syncwarp();
      coulomb_drain(a, st, n, lane);
      __syncwarp();
    }
    if (have) {
      const size_t nn = (size_t)a.natoms;
      add_fix(a.acc + ti, acc_cc, a.st);
      add_fix(a.acc + nn + ti, acc_vdw, a.st);
      add_fix(a.acc + 2 * nn + ti, gx, a.st);
      add_fix(a.acc + 3 * nn + ti, gy, a.st);
      add_fix(a.acc + 4 * nn + ti, gz, a.st);
    }
  }
}

// Per atom (cell order): the fixed-point totals to the per-atom outputs.
__global__ void k_coulomb_finish(const CoulArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.natoms) return;
  const long long* acc = (const long long*)a.acc;
  const size_t n = (size_t)a.natoms;
  const double cc = (double)acc[p] * kFixInv;
  const double vdw = (double)acc[n + p] * kFixInv;
  const float gx = (float)((double)acc[2 * n + p] * kFixInv);
  const float gy = (float)((double)acc[3 * n + p] * kFixInv);
  const float gz = (float)((double)acc[4 * n + p] * kFixInv);
  const int i = a.eatom[p];
  const float qi = a.exlo[p].w;
  a.ecv[2 * i + 0] = 0.5 * (double)qi * cc;
  a.ecv[2 * i + 1] = vdw;   // whole pair energies of the pairs this atom is centre of
  a.dEdqt[i] = (float)cc;
  a.fcv[i] = make_float4(gx, gy, gz, 0.f);
}

// chunk partials: Ecc, Evdw, sum dE/dq~, dipole xyz
__global__ void k_chunk_sum2(const int2* __restrict__ chunk, const double* __restrict__ ecv,
                             const float* __restrict__ dEdqt, const float* __restrict__ q,
                             const double* __restrict__ x, double bohr, double* __restrict__ part) {
  const int2 ch = chunk[blockIdx.x];
  double v[6] = {0, 0, 0, 0, 0, 0};
  for (int i = ch.x + threadIdx.x; i < ch.y; i += blockDim.x) {
    v[0] += ecv[2 * i];
    v[1] += ecv[2 * i + 1];
    v[2] += (double)dEdqt[i];
    const double qq = (double)q[i];
    v[3] += qq * x[3 * i] * bohr;
    v[4] += qq * x[3 * i + 1] * bohr;
    v[5] += qq * x[3 * i + 2] * bohr;
  }
  block_sum_store<6>(v, part + 8 * (size_t)blockIdx.x);
}

__global__ void k_mol_final2(const int32_t* __restrict__ mol_chunk, const double* __restrict__ part,
                             double* __restrict__ molE, double* __restrict__ aux, int nmol) {
  const int m = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (m >= nmol) return;
  const int slot[6] = {0, 1, 2, 3, 4, 5};
  double v[6];
  warp_chunk_sum<6>(mol_chunk, part, m, lane, slot, v);
  if (lane == 0) {
    molE[4 * m + 2] = v[0];
    molE[4 * m + 3] = v[1];
    molE[4 * m + 0] = molE[4 * m + 1] + v[0] + v[1];
    aux[8 * m + 1] = v[2];
    aux[8 * m + 2] = v[3];
    aux[8 * m + 3] = v[4];
    aux[8 * m + 4] = v[5];
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
  const int nsplit = tm_gemm_row_parts(m->desc.precision, m->H);
  k_mlp_finish<<<s->nchunk, 256, 0, ctx->stream>>>(s->d_chunk, s->epart, m->bout, s->row_of_atom,
                                                   s->d_elem, nsplit, s->Mpad, m->k.nele,
                                                   s->d_Eatom, s->d_qraw, s->d_part);
  k_mol_final1<<<tm_div_up(s->nmol, 4), 128, 0, ctx->stream>>>(s->d_mol_chunk, s->d_part,
                                                                 s->d_mol_E, s->d_mol_aux, s->nmol);
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
  a.mol = s->d_mol; a.grid = s->d_egrid; a.cell_start = s->d_ecell_start;
  a.cell_of = s->d_ecell_of_atom; a.blk = s->d_eblk; a.nblk = s->d_neblk;
  a.blk_cap = s->N / 32 + s->ecell_cap + 1; a.ecv = s->d_ecv; a.dEdqt = s->d_dEdq; a.fcv = s->d_fcv;
  a.acc = s->d_cacc; a.natoms = s->N; a.st = ctx->d_status;
  a.ref_periodic = (s->periodic && (flags & TM_F_REFERENCE_PERIODIC_FORCE)) ? 1 : 0;
  a.periodic = s->periodic ? 1 : 0;
  a.ree = k.ree_d;
  a.ree2 = (float)(k.ree_d * k.ree_d);
  a.ree2_lo = a.ree2 * (1.f - kBand);
  a.ree2_hi = a.ree2 * (1.f + kBand);
  a.reach = k.ree_d + s->skin;
  a.reach2 = (float)(a.reach * a.reach) * (1.f + kBand);
  a.pre2 = a.ree2 * (1.f + 2.f * kBand);
  a.inv_bohr = (float)(1.0 / (double)k.bohr);
  a.inv_b2 = (float)(1.0 / ((double)k.bohr * (double)k.bohr));
  a.inv_vdw_width = (float)(1.0 / (double)k.vdw_width);
  a.c_lin = (float)((double)k.zz / (double)k.r_lr + (double)k.yy);
  for (int q = 0; q < 9; ++q) a.lat[q] = s->lat[q];
  a.ortho = s->ortho ? 1 : 0;
  for (int d = 0; d < 3; ++d)   // the periodic Coulomb grid has ee_dims cells per lattice vector
    for (int e = 0; e < 3; ++e) a.cu[3 * d + e] = s->periodic ? s->lat[3 * d + e] / s->ee_dims[d] : 0.0;
  tm_fill_shifts(s, a.sh_hi, a.sh_lo);
  cudaMemsetAsync(s->d_cacc, 0, sizeof(unsigned long long) * 5 * (size_t)s->N, ctx->stream);
  if (s->periodic && !s->ortho)
    k_coulomb<true><<<tm_div_up(a.blk_cap * TM_EE_SPLIT, 4), 128, 0, ctx->stream>>>(a, k);
  else
    k_coulomb<false><<<tm_div_up(a.blk_cap * TM_EE_SPLIT, 4), 128, 0, ctx->stream>>>(a, k);
  k_coulomb_finish<<<tm_div_up(s->N, 256), 256, 0, ctx->stream>>>(a);
  ctx->launches += 2;
  k_chunk_sum2<<<s->nchunk, 256, 0, ctx->stream>>>(s->d_chunk, s->d_ecv, s->d_dEdq, s->d_q,
                                                   s->d_x, 1.889725989, s->d_part);
  k_mol_final2<<<tm_div_up(s->nmol, 4), 128, 0, ctx->stream>>>(s->d_mol_chunk, s->d_part,
                                                                 s->d_mol_E, s->d_mol_aux, s->nmol);
  k_dq<<<tm_div_up(s->N, 256), 256, 0, ctx->stream>>>(s->d_mol, s->d_off, s->d_mol_aux, s->d_dEdq,
                                                      s->N);
  ctx->launches += 4;
  return tm_cuda_check(ctx, cudaGetLastError(), "coulomb");
}
