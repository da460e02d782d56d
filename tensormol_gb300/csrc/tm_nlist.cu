// Cell-list neighbour build, bit-exact with the reference's pair and triple sets.
//
// Reference: MolEmb.Make_NListNaive (C_API/MolEmb.cpp:1180-1251) decides
// membership with sqrt(dx^2+dy^2+dz^2) + 1e-13 < rc in FP64; the Python layer
// (ForceModifiers/Neighbors.py:117-201, 344-470) flattens, builds j<k triples,
// tags elements, lexsorts and numbers slots. Here:
//   * atoms are binned per molecule into cells of edge >= AN1_r_Rc;
//   * one warp per centre atom screens the 27 neighbouring cells with an FP32
//     double-single distance and settles every candidate within 1e-5 (relative,
//     on d^2) of a cutoff with the reference's exact FP64 expression;
//   * accepted neighbours are sorted per centre by (element, reference index),
//     which is the reference's (mol, i, l, j) lexsort order, and stored in
//     fixed-capacity rows (ELL) for the descriptor kernels;
//   * periodic cells use minimum-image search over wrapped cells; each entry
//     carries the image shift whose raster index reproduces the reference's
//     27-image tessellation numbering (ForceModifiers/Periodic.py:131-181).
#include <cuda_runtime.h>

#include "tm_internal.h"

void tm_fill_shifts(const tm_system* s, float hi[27][3], float lo[27][3]);   // tm_desc.cu

namespace {

constexpr float kBand = 1e-5f;   // relative band on d^2 settled in FP64

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---------------------------------------------------------------------------
// positions: FP64 -> double-single, finiteness check
// ---------------------------------------------------------------------------
__global__ void k_positions(const double* __restrict__ x, const int32_t* __restrict__ elem,
                            float4* __restrict__ xhi, float4* __restrict__ xlo, int N,
                            tm_dev_status* st) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double a = x[3 * i], b = x[3 * i + 1], c = x[3 * i + 2];
  if (!isfinite(a) || !isfinite(b) || !isfinite(c)) tm_flag(st, TM_E_NONFINITE, i, 1);
  float ah = (float)a, bh = (float)b, ch = (float)c;
  xhi[i] = make_float4(ah, bh, ch, __int_as_float(elem[i]));
  xlo[i] = make_float4((float)(a - (double)ah), (float)(b - (double)bh), (float)(c - (double)ch), 0.f);
}

// ---------------------------------------------------------------------------
// per-molecule grid set-up (block per molecule)
// ---------------------------------------------------------------------------
__device__ tm_grid grid_from_bbox(double* mn, double* mx, int a0, int a1, double rc, int periodic,
                                  double Lx, double Ly, double Lz, double occ, double cap_a,
                                  double cap_c, int pnx, int pny, int pnz);

// rc: smallest cell edge. occ > 0 sizes open-boundary cells for about occ
// atoms each (Coulomb grid); cap_a * n + cap_c bounds the cells of a molecule.
// Periodic grids take pn[] cells per edge when given, else floor(L / rc).
__global__ void k_grid_setup(const double* __restrict__ x, const int32_t* __restrict__ off,
                             tm_grid* __restrict__ grid, int32_t* __restrict__ ncell_m,
                             double rc, int periodic, double Lx, double Ly, double Lz,
                             double occ, double cap_a, double cap_c, int pnx, int pny, int pnz) {
  const int m = blockIdx.x;
  const int a0 = off[m], a1 = off[m + 1];
  __shared__ double smin[3][32], smax[3][32];
  double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
  for (int a = a0 + threadIdx.x; a < a1; a += blockDim.x) {
    for (int d = 0; d < 3; ++d) {
      double v = x[3 * a + d];
      mn[d] = fmin(mn[d], v);
      mx[d] = fmax(mx[d], v);
    }
  }
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[d] = fmin(mn[d], __shfl_xor_sync(TM_FULL, mn[d], o));
      mx[d] = fmax(mx[d], __shfl_xor_sync(TM_FULL, mx[d], o));
    }
  }
  const int w = threadIdx.x / 32, l = threadIdx.x % 32, nw = blockDim.x / 32;
  if (l == 0)
    for (int d = 0; d < 3; ++d) { smin[d][w] = mn[d]; smax[d][w] = mx[d]; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int d = 0; d < 3; ++d) {
      for (int q = 1; q < nw; ++q) { mn[d] = fmin(mn[d], smin[d][q]); mx[d] = fmax(mx[d], smax[d][q]); }
    }
    grid[m] = grid_from_bbox(mn, mx, a0, a1, rc, periodic, Lx, Ly, Lz, occ, cap_a, cap_c, pnx, pny, pnz);
    ncell_m[m] = grid[m].nx * grid[m].ny * grid[m].nz;
  }
}

// Grid of one molecule from its bounding box (see k_grid_setup for the
// parameters). Open-boundary cells start at rc (or at the occupancy-based size)
// and grow by 1.25x until the molecule has at most cap_a * n + cap_c cells.
__device__ tm_grid grid_from_bbox(double* mn, double* mx, int a0, int a1, double rc, int periodic,
                                  double Lx, double Ly, double Lz, double occ, double cap_a,
                                  double cap_c, int pnx, int pny, int pnz) {
  {
    tm_grid g;
    g.atom_off = a0;
    g.natom = a1 - a0;
    g.periodic = periodic;
    g.pad = 0;
    if (periodic) {
      g.ox = g.oy = g.oz = 0.0;
      g.nx = pnx > 0 ? pnx : max(1, (int)floor(Lx / rc));
      g.ny = pny > 0 ? pny : max(1, (int)floor(Ly / rc));
      g.nz = pnz > 0 ? pnz : max(1, (int)floor(Lz / rc));
      g.cx = Lx / g.nx; g.cy = Ly / g.ny; g.cz = Lz / g.nz;
    } else {
      if (a1 <= a0) { mn[0] = mn[1] = mn[2] = 0.0; mx[0] = mx[1] = mx[2] = 0.0; }
      // non-finite or absurd extents collapse to a single cell (the positions
      // kernel has already flagged them); counts never exceed the cap
      double ext[3];
      for (int d = 0; d < 3; ++d) {
        ext[d] = mx[d] - mn[d];
        if (!(ext[d] >= 0.0 && ext[d] < 1e7)) { ext[d] = 0.0; mn[d] = 0.0; }
      }
      g.ox = mn[0]; g.oy = mn[1]; g.oz = mn[2];
      const double cap = cap_a * (a1 - a0) + cap_c;
      double cs = rc;
      if (occ > 0.0) {
        const double vol = fmax(ext[0], rc) * fmax(ext[1], rc) * fmax(ext[2], rc);
        cs = fmax(rc, cbrt(occ * vol / fmax(1.0, (double)(a1 - a0))));
      }
      for (int it = 0; it < 200; ++it) {
        const double p = (floor(ext[0] / cs) + 1.0) * (floor(ext[1] / cs) + 1.0) * (floor(ext[2] / cs) + 1.0);
        if (p <= cap) break;
        cs *= 1.25;
      }
      g.cx = g.cy = g.cz = cs;
      g.nx = (int)floor(ext[0] / cs) + 1;
      g.ny = (int)floor(ext[1] / cs) + 1;
      g.nz = (int)floor(ext[2] / cs) + 1;
      if ((double)g.nx * g.ny * g.nz > cap) g.nx = g.ny = g.nz = 1;
    }
    g.cell_off = 0;
    return g;
  }
}

// Partial bounding boxes of chunks (<= TM_CHUNK atoms of one molecule) from the
// FP32 hi parts: the grid origin only has to be close to the minimum, since an
// atom a rounding error outside the box is clamped into the edge cell, which
// keeps every pair within the cutoff in adjacent cells.
__global__ void k_cbox_chunks(const int2* __restrict__ chunk, const float4* __restrict__ xhi,
                              float* __restrict__ cbox) {
  const int2 ch = chunk[blockIdx.x];
  float mn[3] = {3e38f, 3e38f, 3e38f}, mx[3] = {-3e38f, -3e38f, -3e38f};
  for (int a = ch.x + threadIdx.x; a < ch.y; a += blockDim.x) {
    const float4 h = xhi[a];
    mn[0] = fminf(mn[0], h.x); mx[0] = fmaxf(mx[0], h.x);
    mn[1] = fminf(mn[1], h.y); mx[1] = fmaxf(mx[1], h.y);
    mn[2] = fminf(mn[2], h.z); mx[2] = fmaxf(mx[2], h.z);
  }
  __shared__ float sh[6][8];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[d] = fminf(mn[d], __shfl_xor_sync(TM_FULL, mn[d], o));
      mx[d] = fmaxf(mx[d], __shfl_xor_sync(TM_FULL, mx[d], o));
    }
    if (l == 0) { sh[d][w] = mn[d]; sh[3 + d][w] = mx[d]; }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int d = 0; d < 3; ++d) {
      for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
        mn[d] = fminf(mn[d], sh[d][q]);
        mx[d] = fmaxf(mx[d], sh[3 + d][q]);
      }
      cbox[8 * blockIdx.x + d] = mn[d];
      cbox[8 * blockIdx.x + 3 + d] = mx[d];
    }
  }
}

// One thread per molecule: combine its chunk boxes (widened by a relative
// 1e-6 + 1e-5 A margin) and set up the grid.
__global__ void k_grid_from_chunks(const float* __restrict__ cbox, const int32_t* __restrict__ mol_chunk,
                                   const int32_t* __restrict__ off, tm_grid* __restrict__ grid,
                                   int32_t* __restrict__ ncell_m, int nmol, double rc, int periodic,
                                   double Lx, double Ly, double Lz, double occ, double cap_a,
                                   double cap_c, int pnx, int pny, int pnz, int32_t* total,
                                   int cap, tm_dev_status* st) {
  // one warp per molecule: lanes reduce the chunk boxes, lane 0 sizes the grid;
  // with one molecule (total != nullptr) it also writes the cell total that
  // k_grid_offsets would
  const int m = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (m >= nmol) return;
  float mnf[3] = {3e38f, 3e38f, 3e38f}, mxf[3] = {-3e38f, -3e38f, -3e38f};
  for (int c = mol_chunk[m] + lane; c < mol_chunk[m + 1]; c += 32)
    for (int d = 0; d < 3; ++d) {
      mnf[d] = fminf(mnf[d], cbox[8 * c + d]);
      mxf[d] = fmaxf(mxf[d], cbox[8 * c + 3 + d]);
    }
  for (int o = 16; o > 0; o >>= 1)
    for (int d = 0; d < 3; ++d) {
      mnf[d] = fminf(mnf[d], __shfl_xor_sync(TM_FULL, mnf[d], o));
      mxf[d] = fmaxf(mxf[d], __shfl_xor_sync(TM_FULL, mxf[d], o));
    }
  if (lane != 0) return;
  double mn[3], mx[3];
  for (int d = 0; d < 3; ++d) {
    mn[d] = (double)mnf[d] - (1e-5 + 1e-6 * fabs((double)mnf[d]));
    mx[d] = (double)mxf[d] + (1e-5 + 1e-6 * fabs((double)mxf[d]));
  }
  const tm_grid g = grid_from_bbox(mn, mx, off[m], off[m + 1], rc, periodic, Lx, Ly, Lz, occ,
                                   cap_a, cap_c, pnx, pny, pnz);
  grid[m] = g;
  ncell_m[m] = g.nx * g.ny * g.nz;
  if (total) {
    *total = g.nx * g.ny * g.nz;
    if (g.nx * g.ny * g.nz > cap) tm_flag(st, TM_E_CAPACITY, g.nx * g.ny * g.nz, 2);
  }
}

__device__ __forceinline__ int cell_coord(double v, double o, double c, int n) {
  int q = (int)floor((v - o) / c);
  return q < 0 ? 0 : (q >= n ? n - 1 : q);
}

// nrm: rows are the directions the cells are sliced along (the lattice
// planes' unit normals of a periodic cell, whose cell spacings g.c* are
// measured along them; the identity for open systems and orthorhombic cells,
// for which the coordinate is the Cartesian one exactly)
__global__ void k_cell_count(const double* __restrict__ x, const int32_t* __restrict__ mol,
                             const tm_grid* __restrict__ grid, int32_t* __restrict__ cnt,
                             int32_t* __restrict__ cell_of, int N, int cap, tm_dev_status* st,
                             const tm_mat3 nrm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const tm_grid g = grid[mol[i]];
  const double xi = x[3 * i], yi = x[3 * i + 1], zi = x[3 * i + 2];
  const double* n = nrm.v;
  int ix = cell_coord(xi * n[0] + yi * n[1] + zi * n[2], g.ox, g.cx, g.nx);
  int iy = cell_coord(xi * n[3] + yi * n[4] + zi * n[5], g.oy, g.cy, g.ny);
  int iz = cell_coord(xi * n[6] + yi * n[7] + zi * n[8], g.oz, g.cz, g.nz);
  int c = g.cell_off + (ix * g.ny + iy) * g.nz + iz;
  if (c < 0 || c >= cap) {   // cannot happen for a valid grid; never index out of range
    tm_flag(st, TM_E_CAPACITY, i, 2);
    c = 0;
  }
  cell_of[i] = c;
  atomicAdd(&cnt[c], 1);
}

__global__ void k_cell_fill(const int32_t* __restrict__ cell_of, const int32_t* __restrict__ start,
                            int32_t* __restrict__ cursor, int32_t* __restrict__ atoms, int N) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int c = cell_of[i];
  atoms[start[c] + atomicAdd(&cursor[c], 1)] = i;
}

// Atom order inside a cell is made deterministic (ascending index).
// Atoms of each cell in ascending index order (the fill used atomics), one
// warp per cell: every atom's rank is the number of smaller indices in the
// cell, counted from a copy (shared memory up to kSortMax atoms, else the
// cell's range of tmp[], for cells that crowding has made very large).
constexpr int kSortMax = 128;
__global__ void __launch_bounds__(128) k_cell_sort(const int32_t* __restrict__ start,
                                                   int32_t* __restrict__ atoms,
                                                   int32_t* __restrict__ tmp,
                                                   const int32_t* __restrict__ ncell, int cap) {
  __shared__ int32_t buf[4][kSortMax];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * 4 + wib;
  if (c >= cap || c >= *ncell) return;
  const int a = start[c], b = start[c + 1], n = b - a;
  if (n <= 1) return;
  if (n <= kSortMax) {
    int32_t* v = buf[wib];
    for (int t = lane; t < n; t += 32) v[t] = atoms[a + t];
    __syncwarp();
    for (int t = lane; t < n; t += 32) {
      const int x = v[t];
      int rank = 0;
      for (int q = 0; q < n; ++q) rank += v[q] < x;
      atoms[a + rank] = x;
    }
  } else {
    for (int t = lane; t < n; t += 32) tmp[a + t] = atoms[a + t];
    __syncwarp();
    for (int t = lane; t < n; t += 32) {
      const int x = tmp[a + t];
      int rank = 0;
      for (int q = 0; q < n; ++q) rank += tmp[a + q] < x;
      atoms[a + rank] = x;
    }
  }
}

// Cell-ordered copies of the double-single positions for the pair kernel;
// the charge slot (lo.w) is filled after the charge network runs.
// Coulomb-grid packing: atoms in cell order with their positions relative to
// the origin of their own cell (FP64 difference rounded once to FP32; w =
// element). The charge (olo.w) is written after the charge network.
// A periodic cell's grid cell (ix, iy, iz) has its origin at
// ix a0/nx + iy a1/ny + iz a2/nz (lat: the lattice vectors as rows).
__global__ void k_ee_pack(const int32_t* __restrict__ order, const double* __restrict__ x,
                          const int32_t* __restrict__ elem, const int32_t* __restrict__ mol,
                          const tm_grid* __restrict__ grid, const int32_t* __restrict__ cell_of,
                          int32_t* __restrict__ pos, float4* __restrict__ ohi, int N,
                          const tm_mat3 lat) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  const int a = order[p];
  pos[a] = p;
  const tm_grid g = grid[mol[a]];
  const int lc = cell_of[a] - g.cell_off;
  const int iz = lc % g.nz, iy = (lc / g.nz) % g.ny, ix = lc / (g.nz * g.ny);
  double o[3];
  if (g.periodic) {
    const double* L = lat.v;
    for (int d = 0; d < 3; ++d)
      o[d] = ix * (L[d] / g.nx) + iy * (L[3 + d] / g.ny) + iz * (L[6 + d] / g.nz);
  } else {
    o[0] = g.ox + ix * g.cx;
    o[1] = g.oy + iy * g.cy;
    o[2] = g.oz + iz * g.cz;
  }
  ohi[p] = make_float4((float)(x[3 * a] - o[0]), (float)(x[3 * a + 1] - o[1]),
                       (float)(x[3 * a + 2] - o[2]), __int_as_float(elem[a]));
}

// Centre blocks of the pair-term kernel: runs of up to 32 consecutive atoms
// (cell order) within one (x, y) column of a molecule's Coulomb grid. The
// order of the table does not matter (every block's sums are exact integer
// additions).
__global__ void k_ee_blocks(const int32_t* __restrict__ order, const int32_t* __restrict__ mol,
                            const tm_grid* __restrict__ grid, const int32_t* __restrict__ cell_of,
                            const int32_t* __restrict__ cell_start, int4* __restrict__ blk,
                            int32_t* __restrict__ nblk, int N, int cap, tm_dev_status* st) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  const int a = order[p];
  const tm_grid g = grid[mol[a]];
  const int c = cell_of[a];
  const int head = c - (c - g.cell_off) % g.nz;
  const int cs = cell_start[head];
  if ((p - cs) % 32) return;
  const int ce = cell_start[head + g.nz];
  const int slot = atomicAdd(nblk, 1);
  if (slot < cap) blk[slot] = make_int4(head, p, min(p + 32, ce), 0);
  else tm_flag(st, TM_E_CAPACITY, slot, 2);
}

// First cell of every molecule's grid (exclusive prefix sum of the cell
// counts) and the total, by one block of 256 threads: thread t sums a
// contiguous run of molecules, the run sums are scanned in shared memory, and
// each thread then writes its run's offsets (one fixed order of additions).
__global__ void k_grid_offsets(tm_grid* __restrict__ grid, const int32_t* __restrict__ ncell_m,
                               int nmol, int32_t* __restrict__ total, int cap, tm_dev_status* st) {
  __shared__ int part[256];
  const int t = threadIdx.x;
  const int per = (nmol + 255) / 256;
  const int m0 = min(t * per, nmol), m1 = min(m0 + per, nmol);
  int sum = 0;
  for (int m = m0; m < m1; ++m) sum += ncell_m[m];
  part[t] = sum;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {
    const int v = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int acc = part[t] - sum;   // exclusive
  for (int m = m0; m < m1; ++m) {
    grid[m].cell_off = acc;
    acc += ncell_m[m];
  }
  if (t == 255) {
    *total = part[255];
    if (part[255] > cap) tm_flag(st, TM_E_CAPACITY, part[255], 2);
  }
}

// ---------------------------------------------------------------------------
// exclusive scan (int32 / int64), three passes
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_scan_blocks(const T* __restrict__ in, T* __restrict__ out, T* __restrict__ bsum,
                              int64_t n) {
  __shared__ T s[1024];
  const int64_t base = (int64_t)blockIdx.x * 4096;
  T v[4];
  T tsum = 0;
  for (int q = 0; q < 4; ++q) {
    int64_t idx = base + threadIdx.x * 4 + q;
    v[q] = idx < n ? in[idx] : (T)0;
    tsum += v[q];
  }
  s[threadIdx.x] = tsum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    T t = threadIdx.x >= o ? s[threadIdx.x - o] : (T)0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  T run = s[threadIdx.x] - tsum;
  for (int q = 0; q < 4; ++q) {
    int64_t idx = base + threadIdx.x * 4 + q;
    if (idx < n) out[idx] = run;
    run += v[q];
  }
  if (threadIdx.x == 1023) bsum[blockIdx.x] = s[1023];
}

template <typename T>
__global__ void k_scan_top(T* __restrict__ bsum, int nb, T* __restrict__ total) {
  __shared__ T s[1024];
  // nb <= 1024 * 4
  T v[4];
  T tsum = 0;
  for (int q = 0; q < 4; ++q) {
    int idx = threadIdx.x * 4 + q;
    v[q] = idx < nb ? bsum[idx] : (T)0;
    tsum += v[q];
  }
  s[threadIdx.x] = tsum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    T t = threadIdx.x >= o ? s[threadIdx.x - o] : (T)0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  T run = s[threadIdx.x] - tsum;
  for (int q = 0; q < 4; ++q) {
    int idx = threadIdx.x * 4 + q;
    if (idx < nb) bsum[idx] = run;
    run += v[q];
  }
  if (threadIdx.x == 1023 && total) *total = s[1023];
}

template <typename T>
__global__ void k_scan_add(T* __restrict__ out, const T* __restrict__ bsum, int64_t n) {
  int64_t idx = (int64_t)blockIdx.x * 4096 + threadIdx.x;
  T add = bsum[blockIdx.x];
  for (int q = 0; q < 4; ++q, idx += 1024)
    if (idx < n) out[idx] += add;
}

// ---------------------------------------------------------------------------
// neighbour build: one warp per centre atom
// ---------------------------------------------------------------------------
struct NbrArgs {
  const double* x;
  const float4* xhi;
  const float4* xlo;
  const int32_t* mol;
  const int32_t* elem;
  const tm_grid* grid;
  const int32_t* cell_of;
  const int32_t* cell_start;
  const int32_t* cell_atoms;
  int32_t* cnt_r;
  int32_t* cnt_a;
  uint32_t* nbr_r;
  uint32_t* nbr_a;
  int32_t* need;      // [2] max counts seen (radial, angular)
  int N, KR, KA;
  double rr, ra;      // radial / angular cutoffs (FP64, exact test)
  float rr2_lo, rr2_hi, ra2_lo, ra2_hi;
  double lat[9];
};

__device__ __forceinline__ uint64_t nbr_key(int elem, int r, int local) {
  return ((uint64_t)elem << 37) | ((uint64_t)tm_ref_image_index(r) << 32) | (uint32_t)local;
}
__device__ __forceinline__ int ref_to_raster(int ref) {
  return ref == 0 ? TM_IMG_SELF : (ref <= TM_IMG_SELF ? ref - 1 : ref);
}

template <bool PERIODIC>
__global__ void __launch_bounds__(128) k_nbr_build(const NbrArgs a) {
  extern __shared__ uint64_t sh_keys[];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * (blockDim.x >> 5) + wib;
  uint64_t* kr = sh_keys + (size_t)wib * (a.KR + a.KA);
  uint64_t* ka = kr + a.KR;
  if (w >= a.N) return;
  // centres in cell order: the warps of a block share their candidate cells
  const int i = a.cell_atoms[w];
  const int m = a.mol[i];
  const tm_grid g = a.grid[m];
  const float4 hi = a.xhi[i], lo = a.xlo[i];
  const double xi = a.x[3 * i], yi = a.x[3 * i + 1], zi = a.x[3 * i + 2];
  const int lc = a.cell_of[i] - g.cell_off;
  const int iz = lc % g.nz, iy = (lc / g.nz) % g.ny, ix = lc / (g.nz * g.ny);
  int nr = 0, na = 0;
  if constexpr (!PERIODIC) {
    // Open boundary: the three cells of each of the 9 (x, y) columns are one
    // contiguous run of atoms (cell order). Lanes 0..8 load the 9 runs'
    // bounds at once, the runs are laid end to end as one candidate index
    // space, and each iteration takes two chunks of 32 candidates with their
    // loads in flight together (the rows are sorted at the end, so the order
    // in which candidates are met does not matter).
    int ct0 = 0, clen = 0;
    if (lane < 9) {
      const int jx = ix + lane / 3 - 1, jy = iy + lane % 3 - 1;
      if (jx >= 0 && jx < g.nx && jy >= 0 && jy < g.ny) {
        const int cbase = g.cell_off + (jx * g.ny + jy) * g.nz;
        ct0 = a.cell_start[cbase + max(iz - 1, 0)];
        clen = a.cell_start[cbase + min(iz + 1, g.nz - 1) + 1] - ct0;
      }
    }
    int incl = clen;
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) {
      const int v = __shfl_up_sync(TM_FULL, incl, o);
      if (lane >= o) incl += v;
    }
    int pre[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) pre[q] = __shfl_sync(TM_FULL, incl, q);
    const int total = pre[8];
    const int excl = incl - clen;
    // candidate f of the flattened runs: its run k and its atom slot t
    auto slot = [&](int f) {
      int k = 0;
#pragma unroll
      for (int q = 0; q < 9; ++q) k += f >= pre[q] ? 1 : 0;
      k = min(k, 8);
      return __shfl_sync(TM_FULL, ct0, k) + (f - __shfl_sync(TM_FULL, excl, k));
    };
    auto take = [&](bool valid, int j, float4 hj, float4 lj) {
      bool in_r = false, in_a = false;
      uint64_t key = 0;
      if (valid && j != i) {
        const float dx = ds_sub(hi.x, lo.x, hj.x, lj.x);
        const float dy = ds_sub(hi.y, lo.y, hj.y, lj.y);
        const float dz = ds_sub(hi.z, lo.z, hj.z, lj.z);
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 <= a.rr2_hi) {
          const double xj = a.x[3 * j], yj = a.x[3 * j + 1], zj = a.x[3 * j + 2];
          in_r = d2 < a.rr2_lo ? true : tm_exact_within(xi, yi, zi, xj, yj, zj, a.rr);
          if (in_r) in_a = d2 < a.ra2_lo ? true
                           : (d2 <= a.ra2_hi ? tm_exact_within(xi, yi, zi, xj, yj, zj, a.ra) : false);
          key = nbr_key(__float_as_int(hj.w), TM_IMG_SELF, j - g.atom_off);
        }
      }
      const unsigned mr = __ballot_sync(TM_FULL, in_r);
      const unsigned ma = __ballot_sync(TM_FULL, in_a);
      if (in_r) {
        const int p = nr + __popc(mr & lanemask_lt());
        if (p < a.KR) kr[p] = key;
      }
      if (in_a) {
        const int p = na + __popc(ma & lanemask_lt());
        if (p < a.KA) ka[p] = key;
      }
      nr += __popc(mr);
      na += __popc(ma);
    };
    for (int f0 = 0; f0 < total; f0 += 64) {
      const int fa = f0 + lane, fb = f0 + 32 + lane;
      const bool va = fa < total, vb = fb < total;
      const int ta = slot(fa), tb = slot(fb);
      const int ja = va ? a.cell_atoms[ta] : i, jb = vb ? a.cell_atoms[tb] : i;
      const float4 ha = a.xhi[ja], la = a.xlo[ja], hb = a.xhi[jb], lb = a.xlo[jb];
      take(va, ja, ha, la);
      take(vb, jb, hb, lb);
    }
  }
  // the three cells of a z column without a periodic wrap are one contiguous
  // run of atoms (cell order); a wrapped column is taken cell by cell
  const bool zrun = !PERIODIC || (iz >= 1 && iz + 1 < g.nz);
  for (int ox = -1; ox <= 1 && PERIODIC; ++ox) {
    for (int oy = -1; oy <= 1; ++oy) {
      for (int oz = zrun ? 0 : -1; oz <= (zrun ? 0 : 1); ++oz) {
        int jx = ix + ox, jy = iy + oy, jz = iz + oz, sx = 0, sy = 0, sz = 0;
        if (PERIODIC) {
          if (jx < 0) { jx += g.nx; sx = -1; } else if (jx >= g.nx) { jx -= g.nx; sx = 1; }
          if (jy < 0) { jy += g.ny; sy = -1; } else if (jy >= g.ny) { jy -= g.ny; sy = 1; }
          if (jz < 0) { jz += g.nz; sz = -1; } else if (jz >= g.nz) { jz -= g.nz; sz = 1; }
        } else {
          if (jx < 0 || jx >= g.nx || jy < 0 || jy >= g.ny) continue;
        }
        const int cbase = g.cell_off + (jx * g.ny + jy) * g.nz;
        const int c0 = cbase + (zrun ? max(iz - 1, 0) : jz);
        const int c1 = cbase + (zrun ? min(iz + 1, g.nz - 1) : jz);
        const int r = 9 * (sx + 1) + 3 * (sy + 1) + (sz + 1);
        // shift added to the neighbour: s = sx*a0 + sy*a1 + sz*a2
        double shx = 0, shy = 0, shz = 0;
        float shx_h = 0, shy_h = 0, shz_h = 0, shx_l = 0, shy_l = 0, shz_l = 0;
        if (PERIODIC) {
          shx = sx * a.lat[0] + sy * a.lat[3] + sz * a.lat[6];
          shy = sx * a.lat[1] + sy * a.lat[4] + sz * a.lat[7];
          shz = sx * a.lat[2] + sy * a.lat[5] + sz * a.lat[8];
          shx_h = (float)shx; shy_h = (float)shy; shz_h = (float)shz;
          shx_l = (float)(shx - shx_h); shy_l = (float)(shy - shy_h); shz_l = (float)(shz - shz_h);
        }
        const int t0 = a.cell_start[c0], t1 = a.cell_start[c1 + 1];
        for (int tb = t0; tb < t1; tb += 32) {
          const int t = tb + lane;
          bool in_r = false, in_a = false;
          uint64_t key = 0;
          if (t < t1) {
            const int j = a.cell_atoms[t];
            if (!(j == i && r == TM_IMG_SELF)) {
              const float4 hj = a.xhi[j], lj = a.xlo[j];
              float dx, dy, dz;
              if (PERIODIC) {
                dx = ds_sub_shift(hi.x, lo.x, hj.x, lj.x, shx_h, shx_l);
                dy = ds_sub_shift(hi.y, lo.y, hj.y, lj.y, shy_h, shy_l);
                dz = ds_sub_shift(hi.z, lo.z, hj.z, lj.z, shz_h, shz_l);
              } else {
                dx = ds_sub(hi.x, lo.x, hj.x, lj.x);
                dy = ds_sub(hi.y, lo.y, hj.y, lj.y);
                dz = ds_sub(hi.z, lo.z, hj.z, lj.z);
              }
              const float d2 = dx * dx + dy * dy + dz * dz;
              if (d2 <= a.rr2_hi) {
                double xj = a.x[3 * j], yj = a.x[3 * j + 1], zj = a.x[3 * j + 2];
                if (PERIODIC) {
                  xj = tm_image_coord(xj, sx, sy, sz, a.lat[0], a.lat[3], a.lat[6]);
                  yj = tm_image_coord(yj, sx, sy, sz, a.lat[1], a.lat[4], a.lat[7]);
                  zj = tm_image_coord(zj, sx, sy, sz, a.lat[2], a.lat[5], a.lat[8]);
                }
                in_r = d2 < a.rr2_lo ? true : tm_exact_within(xi, yi, zi, xj, yj, zj, a.rr);
                if (in_r) in_a = d2 < a.ra2_lo ? true
                                 : (d2 <= a.ra2_hi ? tm_exact_within(xi, yi, zi, xj, yj, zj, a.ra)
                                                   : false);
                key = nbr_key(__float_as_int(hj.w), r, j - g.atom_off);
              }
            }
          }
          const unsigned mr = __ballot_sync(TM_FULL, in_r);
          const unsigned ma = __ballot_sync(TM_FULL, in_a);
          if (in_r) {
            int p = nr + __popc(mr & lanemask_lt());
            if (p < a.KR) kr[p] = key;
          }
          if (in_a) {
            int p = na + __popc(ma & lanemask_lt());
            if (p < a.KA) ka[p] = key;
          }
          nr += __popc(mr);
          na += __popc(ma);
        }
      }
    }
  }
  __syncwarp();
  if (nr > a.KR || na > a.KA) {
    if (lane == 0) {
      atomicMax(&a.need[0], nr);
      atomicMax(&a.need[1], na);
    }
  }
  const int cr = min(nr, a.KR), ca = min(na, a.KA);
  // rank sort (keys are unique) and write packed entries
  for (int p = lane; p < cr; p += 32) {
    const uint64_t kp = kr[p];
    int rank = 0;
    for (int q = 0; q < cr; ++q) rank += kr[q] < kp;
    const int r = ref_to_raster((int)((kp >> 32) & 31));
    a.nbr_r[(size_t)i * a.KR + rank] = tm_pack((uint32_t)(g.atom_off + (int)(kp & 0xffffffffu)), r);
  }
  for (int p = lane; p < ca; p += 32) {
    const uint64_t kp = ka[p];
    int rank = 0;
    for (int q = 0; q < ca; ++q) rank += ka[q] < kp;
    const int r = ref_to_raster((int)((kp >> 32) & 31));
    a.nbr_a[(size_t)i * a.KA + rank] = tm_pack((uint32_t)(g.atom_off + (int)(kp & 0xffffffffu)), r);
  }
  if (lane == 0) {
    a.cnt_r[i] = cr;
    a.cnt_a[i] = ca;
  }
}

// Reverse edge index: for entry s of centre i (neighbour j at image r),
// the position of i (at image 26 - r) in j's list.
// One launch for both lists: warps [0, N) take the radial rows, [N, 2N) the
// angular rows.
__global__ void k_nbr_reverse(const uint32_t* __restrict__ nbr_r, const int32_t* __restrict__ cnt_r,
                              int32_t* __restrict__ rev_r, int KR,
                              const uint32_t* __restrict__ nbr_a, const int32_t* __restrict__ cnt_a,
                              int32_t* __restrict__ rev_a, int KA, const int32_t* __restrict__ elem,
                              const int32_t* __restrict__ mol, const int32_t* __restrict__ off,
                              int N) {
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * (blockDim.x >> 5) + wib;
  if (w >= 2 * N) return;
  const bool ang = w >= N;
  const int i = ang ? w - N : w;
  const uint32_t* nbr = ang ? nbr_a : nbr_r;
  const int32_t* cnt = ang ? cnt_a : cnt_r;
  int32_t* rev = ang ? rev_a : rev_r;
  const int K = ang ? KA : KR;
  const int ci = cnt[i];
  const int ei = elem[i];
  const int li = i - off[mol[i]];
  for (int s = lane; s < ci; s += 32) {
    const uint32_t e = nbr[(size_t)i * K + s];
    const int j = (int)tm_atom(e);
    const int rj = TM_IMG_SELF * 2 - tm_img(e);
    const uint64_t want = nbr_key(ei, rj, li);
    const int cj = cnt[j];
    const int jo = off[mol[j]];
    int lo = 0, hi = cj - 1, found = -1;
    while (lo <= hi) {
      const int mid = (lo + hi) >> 1;
      const uint32_t q = nbr[(size_t)j * K + mid];
      const int qa = (int)tm_atom(q);
      const uint64_t kq = nbr_key(elem[qa], tm_img(q), qa - jo);
      if (kq == want) { found = mid; break; }
      if (kq < want) lo = mid + 1; else hi = mid - 1;
    }
    rev[(size_t)i * K + s] = found < 0 ? -1 : j * K + found;
  }
}

// ---------------------------------------------------------------------------
// export in the reference's layout
// ---------------------------------------------------------------------------
__global__ void k_export_sizes(const int32_t* __restrict__ cnt_r, const int32_t* __restrict__ cnt_a,
                               int64_t* __restrict__ pr, int64_t* __restrict__ pt, int N) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  pr[i] = cnt_r[i];
  const int64_t c = cnt_a[i];
  pt[i] = c * (c - 1) / 2;
}

struct ExportArgs {
  const uint32_t* nbr_r;
  const uint32_t* nbr_a;
  const int32_t* cnt_r;
  const int32_t* cnt_a;
  const int32_t* elem;
  const int32_t* mol;
  const int32_t* off;
  const int64_t* pr;   // exclusive offsets
  const int64_t* pt;
  int64_t* radp;       // [P][4]
  int64_t* milj;       // [P][4]
  int64_t* angt;       // [T][5]
  int64_t* miljk;      // [T][4]
  int N, KR, KA, nele, nreal_stride;
  int elepair[TM_MAX_ELE][TM_MAX_ELE];
};

__device__ __forceinline__ int64_t ref_index(uint32_t e, int jo, int nreal) {
  return (int64_t)tm_ref_image_index(tm_img(e)) * nreal + ((int)tm_atom(e) - jo);
}

__global__ void k_export_lists(const ExportArgs a) {
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + wib;
  if (i >= a.N) return;
  const int m = a.mol[i];
  const int jo = a.off[m];
  const int li = i - jo;
  const int nreal = a.nreal_stride > 0 ? a.nreal_stride : (a.off[m + 1] - jo);
  // radial: segment starts per element
  const int cr = a.cnt_r[i];
  int seg[TM_MAX_ELE + 1];
  for (int e = 0; e < a.nele; ++e) {
    int c = 0;
    for (int s = lane; s < cr; s += 32) c += a.elem[tm_atom(a.nbr_r[(size_t)i * a.KR + s])] == e;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(TM_FULL, c, o);
    seg[e] = c;
  }
  {
    int acc = 0;
    for (int e = 0; e < a.nele; ++e) { int c = seg[e]; seg[e] = acc; acc += c; }
    seg[a.nele] = acc;
  }
  if (a.radp || a.milj) {
    const int64_t base = a.pr[i];
    for (int s = lane; s < cr; s += 32) {
      const uint32_t e = a.nbr_r[(size_t)i * a.KR + s];
      const int l = a.elem[tm_atom(e)];
      const int64_t row = base + s;
      if (a.radp) {
        a.radp[row * 4 + 0] = m; a.radp[row * 4 + 1] = li;
        a.radp[row * 4 + 2] = ref_index(e, jo, nreal); a.radp[row * 4 + 3] = l;
      }
      if (a.milj) {
        a.milj[row * 4 + 0] = m; a.milj[row * 4 + 1] = li;
        a.milj[row * 4 + 2] = l; a.milj[row * 4 + 3] = s - seg[l];
      }
    }
  }
  if (!(a.angt || a.miljk)) return;
  // angular: element segments of the angular list
  const int ca = a.cnt_a[i];
  for (int e = 0; e < a.nele; ++e) {
    int c = 0;
    for (int s = lane; s < ca; s += 32) c += a.elem[tm_atom(a.nbr_a[(size_t)i * a.KA + s])] == e;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(TM_FULL, c, o);
    seg[e] = c;
  }
  {
    int acc = 0;
    for (int e = 0; e < a.nele; ++e) { int c = seg[e]; seg[e] = acc; acc += c; }
    seg[a.nele] = acc;
  }
  int64_t row0 = a.pt[i];
  for (int ea = 0; ea < a.nele; ++ea) {
    for (int eb = ea; eb < a.nele; ++eb) {
      const int na_ = seg[ea + 1] - seg[ea], nb_ = seg[eb + 1] - seg[eb];
      const int64_t npair = ea < eb ? (int64_t)na_ * nb_ : (int64_t)na_ * (na_ - 1) / 2;
      const int l = a.elepair[ea][eb];
      for (int64_t t = lane; t < npair; t += 32) {
        int pa, pb;
        if (ea < eb) {
          pb = (int)(t / na_);
          pa = (int)(t % na_);
        } else {
          // t = b(b-1)/2 + a with 0 <= a < b
          int b = (int)((1.0 + sqrt(1.0 + 8.0 * (double)t)) * 0.5);
          while ((int64_t)b * (b - 1) / 2 > t) --b;
          while ((int64_t)(b + 1) * b / 2 <= t) ++b;
          pb = b;
          pa = (int)(t - (int64_t)b * (b - 1) / 2);
        }
        const uint32_t ej = a.nbr_a[(size_t)i * a.KA + seg[ea] + pa];
        const uint32_t ek = a.nbr_a[(size_t)i * a.KA + seg[eb] + pb];
        const int64_t row = row0 + t;
        if (a.angt) {
          a.angt[row * 5 + 0] = m; a.angt[row * 5 + 1] = li;
          a.angt[row * 5 + 2] = ref_index(ej, jo, nreal);
          a.angt[row * 5 + 3] = ref_index(ek, jo, nreal);
          a.angt[row * 5 + 4] = l;
        }
        if (a.miljk) {
          a.miljk[row * 4 + 0] = m; a.miljk[row * 4 + 1] = li;
          a.miljk[row * 4 + 2] = l; a.miljk[row * 4 + 3] = t;
        }
      }
      row0 += npair;
    }
  }
}

// Coulomb pair list (materialised only for export / the plain path).
struct EEArgs {
  const double* x;
  const float4* xhi;
  const float4* xlo;
  const int32_t* mol;
  const tm_grid* grid;
  const int32_t* cell_of;
  const int32_t* cell_start;
  const int32_t* cell_atoms;
  const int64_t* offs;    // fill pass: exclusive offsets per centre
  int64_t* count;         // count pass: per centre
  int64_t* out;           // [Pee][3]
  int N;
  double ree;
  float ree2_lo, ree2_hi;
  double lat[9];
  int periodic;
};

template <bool FILL>
__global__ void __launch_bounds__(128) k_ee_pairs(const EEArgs a) {
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + wib;
  if (i >= a.N) return;
  const int m = a.mol[i];
  const tm_grid g = a.grid[m];
  const float4 hi = a.xhi[i], lo = a.xlo[i];
  const double xi = a.x[3 * i], yi = a.x[3 * i + 1], zi = a.x[3 * i + 2];
  const int lc = a.cell_of[i] - g.cell_off;
  const int iz = lc % g.nz, iy = (lc / g.nz) % g.ny, ix = lc / (g.nz * g.ny);
  // periodic: at most one wrap per axis (R <= n; edges are >= 2 * cutoff)
  const int Rx = a.periodic ? min((int)ceil(a.ree / g.cx), g.nx) : (int)ceil(a.ree / g.cx);
  const int Ry = a.periodic ? min((int)ceil(a.ree / g.cy), g.ny) : (int)ceil(a.ree / g.cy);
  const int Rz = a.periodic ? min((int)ceil(a.ree / g.cz), g.nz) : (int)ceil(a.ree / g.cz);
  const int nreal = g.natom;
  int64_t n = 0;
  int64_t base = FILL ? a.offs[i] : 0;
  for (int ox = -Rx; ox <= Rx; ++ox) {
    for (int oy = -Ry; oy <= Ry; ++oy) {
      for (int oz = -Rz; oz <= Rz; ++oz) {
        int jx = ix + ox, jy = iy + oy, jz = iz + oz, sx = 0, sy = 0, sz = 0;
        if (a.periodic) {
          if (jx < 0) { jx += g.nx; sx = -1; } else if (jx >= g.nx) { jx -= g.nx; sx = 1; }
          if (jy < 0) { jy += g.ny; sy = -1; } else if (jy >= g.ny) { jy -= g.ny; sy = 1; }
          if (jz < 0) { jz += g.nz; sz = -1; } else if (jz >= g.nz) { jz -= g.nz; sz = 1; }
        } else if (jx < 0 || jx >= g.nx || jy < 0 || jy >= g.ny || jz < 0 || jz >= g.nz) {
          continue;
        }
        const int c = g.cell_off + (jx * g.ny + jy) * g.nz + jz;
        const int r = 9 * (sx + 1) + 3 * (sy + 1) + (sz + 1);
        double shx = 0, shy = 0, shz = 0;
        if (a.periodic) {
          shx = sx * a.lat[0] + sy * a.lat[3] + sz * a.lat[6];
          shy = sx * a.lat[1] + sy * a.lat[4] + sz * a.lat[7];
          shz = sx * a.lat[2] + sy * a.lat[5] + sz * a.lat[8];
        }
        const float shx_h = (float)shx, shy_h = (float)shy, shz_h = (float)shz;
        const float shx_l = (float)(shx - shx_h), shy_l = (float)(shy - shy_h), shz_l = (float)(shz - shz_h);
        const int t0 = a.cell_start[c], t1 = a.cell_start[c + 1];
        for (int tb = t0; tb < t1; tb += 32) {
          const int t = tb + lane;
          bool ok = false;
          int j = 0;
          if (t < t1) {
            j = a.cell_atoms[t];
            // open: i < j only (DoPerms = 0); periodic: every other atom/image
            const bool cand = a.periodic ? !(j == i && r == TM_IMG_SELF) : (j > i);
            if (cand) {
              const float4 hj = a.xhi[j], lj = a.xlo[j];
              const float dx = ds_sub_shift(hi.x, lo.x, hj.x, lj.x, shx_h, shx_l);
              const float dy = ds_sub_shift(hi.y, lo.y, hj.y, lj.y, shy_h, shy_l);
              const float dz = ds_sub_shift(hi.z, lo.z, hj.z, lj.z, shz_h, shz_l);
              const float d2 = dx * dx + dy * dy + dz * dz;
              if (d2 < a.ree2_lo) ok = true;
              else if (d2 <= a.ree2_hi) {
                double xj = a.x[3 * j], yj = a.x[3 * j + 1], zj = a.x[3 * j + 2];
                if (a.periodic) {
                  xj = tm_image_coord(xj, sx, sy, sz, a.lat[0], a.lat[3], a.lat[6]);
                  yj = tm_image_coord(yj, sx, sy, sz, a.lat[1], a.lat[4], a.lat[7]);
                  zj = tm_image_coord(zj, sx, sy, sz, a.lat[2], a.lat[5], a.lat[8]);
                }
                ok = tm_exact_within(xi, yi, zi, xj, yj, zj, a.ree);
              }
            }
          }
          const unsigned mk = __ballot_sync(TM_FULL, ok);
          if (FILL && ok) {
            const int64_t row = base + n + __popc(mk & lanemask_lt());
            a.out[row * 3 + 0] = m;
            a.out[row * 3 + 1] = i - g.atom_off;
            a.out[row * 3 + 2] = (int64_t)tm_ref_image_index(r) * nreal + (j - g.atom_off);
          }
          n += __popc(mk);
        }
      }
    }
  }
  if (!FILL && lane == 0) a.count[i] = n;
}

template <typename T>
int scan_exclusive(tm_ctx* ctx, const T* in, T* out, int64_t n, T* total_dev,
                   T* scratch = nullptr) {
  const int64_t nb = (n + 4095) / 4096;
  if (nb > 4096) return tm_fail(ctx, TM_E_ARG, "scan too large");
  // scratch (4096 entries) keeps the per-step scans free of allocations
  T* bsum = scratch;
  if (!bsum && tm_alloc(ctx, (void**)&bsum, sizeof(T) * (size_t)(nb > 0 ? nb : 1))) return TM_E_CUDA;
  if (n > 0 && nb == 1) {
    // one block: its exclusive scan is the result and its sum the total
    k_scan_blocks<T><<<1, 1024, 0, ctx->stream>>>(in, out, total_dev ? total_dev : bsum, n);
    ctx->launches += 1;
  } else if (n > 0) {
    k_scan_blocks<T><<<(unsigned)nb, 1024, 0, ctx->stream>>>(in, out, bsum, n);
    k_scan_top<T><<<1, 1024, 0, ctx->stream>>>(bsum, (int)nb, total_dev);
    k_scan_add<T><<<(unsigned)nb, 1024, 0, ctx->stream>>>(out, bsum, n);
    ctx->launches += 3;
  }
  int rc = tm_cuda_check(ctx, cudaGetLastError(), "scan");
  if (!scratch) tm_free(ctx, bsum, sizeof(T) * (size_t)(nb > 0 ? nb : 1));
  return rc;
}

NbrArgs make_nbr_args(tm_system* s, int32_t* need) {
  const tm_consts& k = s->model->k;
  NbrArgs a;
  a.x = s->d_x; a.xhi = s->d_xhi; a.xlo = s->d_xlo; a.mol = s->d_mol; a.elem = s->d_elem;
  a.grid = s->d_grid; a.cell_of = s->d_cell_of_atom; a.cell_start = s->d_cell_start;
  a.cell_atoms = s->d_cell_atoms; a.cnt_r = s->d_cnt_r; a.cnt_a = s->d_cnt_a;
  a.nbr_r = s->d_nbr_r; a.nbr_a = s->d_nbr_a; a.need = need;
  a.N = s->N; a.KR = s->KR; a.KA = s->KA;
  a.rr = k.r_rc_d; a.ra = k.a_rc_d;
  a.rr2_lo = (float)(k.r_rc_d * k.r_rc_d) * (1.f - kBand);
  a.rr2_hi = (float)(k.r_rc_d * k.r_rc_d) * (1.f + kBand);
  a.ra2_lo = (float)(k.a_rc_d * k.a_rc_d) * (1.f - kBand);
  a.ra2_hi = (float)(k.a_rc_d * k.a_rc_d) * (1.f + kBand);
  for (int q = 0; q < 9; ++q) a.lat[q] = s->lat[q];
  return a;
}

// Exact rows from the candidate rows: the same FP32 screen + FP64 membership
// rule as k_nbr_build, applied to each candidate in its (sorted) order, so
// the rows equal a fresh build as long as no atom has moved more than half the
// skin since the candidates were built. Also records the largest squared
// displacement since then (as the bits of a non-negative double).
struct FiltArgs {
  const double* x;
  const double* x0;         // positions at the candidate build
  const float4* xhi;
  const float4* xlo;
  const uint32_t* cand;
  const int32_t* ccnt;
  int32_t* cnt_r;
  int32_t* cnt_a;
  uint32_t* nbr_r;
  uint32_t* nbr_a;
  int32_t* need;
  unsigned long long* disp;
  int N, KC, KR, KA, periodic;
  double rr, ra;
  float rr2_lo, rr2_hi, ra2_lo, ra2_hi;
  double lat[9];
  double binv[9];
  int ortho;
  float sh_hi[27][3], sh_lo[27][3];
};

__global__ void __launch_bounds__(128) k_nbr_filter(const FiltArgs a) {
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= a.N) return;
  const float4 hi = a.xhi[i], lo = a.xlo[i];
  const double xi = a.x[3 * i], yi = a.x[3 * i + 1], zi = a.x[3 * i + 2];
  const int cc = a.ccnt[i];
  int nr = 0, na = 0;
  for (int base = 0; base < cc; base += 32) {
    const int t = base + lane;
    bool in_r = false, in_a = false;
    uint32_t e = 0;
    if (t < cc) {
      e = a.cand[(size_t)i * a.KC + t];
      const int j = (int)tm_atom(e), r = tm_img(e);
      const float4 hj = a.xhi[j], lj = a.xlo[j];
      const float dx = ds_sub_shift(hi.x, lo.x, hj.x, lj.x, a.sh_hi[r][0], a.sh_lo[r][0]);
      const float dy = ds_sub_shift(hi.y, lo.y, hj.y, lj.y, a.sh_hi[r][1], a.sh_lo[r][1]);
      const float dz = ds_sub_shift(hi.z, lo.z, hj.z, lj.z, a.sh_hi[r][2], a.sh_lo[r][2]);
      const float d2 = dx * dx + dy * dy + dz * dz;
      if (d2 <= a.rr2_hi) {
        double xj = a.x[3 * j], yj = a.x[3 * j + 1], zj = a.x[3 * j + 2];
        if (a.periodic) {
          int sx, sy, sz;
          tm_img_ijk(r, sx, sy, sz);
          xj = tm_image_coord(xj, sx, sy, sz, a.lat[0], a.lat[3], a.lat[6]);
          yj = tm_image_coord(yj, sx, sy, sz, a.lat[1], a.lat[4], a.lat[7]);
          zj = tm_image_coord(zj, sx, sy, sz, a.lat[2], a.lat[5], a.lat[8]);
        }
        in_r = d2 < a.rr2_lo ? true : tm_exact_within(xi, yi, zi, xj, yj, zj, a.rr);
        if (in_r) in_a = d2 < a.ra2_lo ? true
                         : (d2 <= a.ra2_hi ? tm_exact_within(xi, yi, zi, xj, yj, zj, a.ra) : false);
      }
    }
    const unsigned mr = __ballot_sync(TM_FULL, in_r);
    const unsigned ma = __ballot_sync(TM_FULL, in_a);
    if (in_r) {
      const int p = nr + __popc(mr & lanemask_lt());
      if (p < a.KR) a.nbr_r[(size_t)i * a.KR + p] = e;
    }
    if (in_a) {
      const int p = na + __popc(ma & lanemask_lt());
      if (p < a.KA) a.nbr_a[(size_t)i * a.KA + p] = e;
    }
    nr += __popc(mr);
    na += __popc(ma);
  }
  if (lane == 0) {
    if (nr > a.KR || na > a.KA) {
      atomicMax(&a.need[0], nr);
      atomicMax(&a.need[1], na);
    }
    a.cnt_r[i] = min(nr, a.KR);
    a.cnt_a[i] = min(na, a.KA);
    double d2 = 0.0;
    double u[3];
    for (int d = 0; d < 3; ++d) u[d] = a.x[3 * i + d] - a.x0[3 * i + d];
    if (a.periodic && a.ortho) {   // wrapped into the cell since the build: nearest image
      for (int d = 0; d < 3; ++d) {
        const double L = a.lat[4 * d];
        u[d] -= L * rint(u[d] / L);
      }
    } else if (a.periodic) {       // the same in fractional coordinates
      double f[3];
      for (int d = 0; d < 3; ++d) {
        f[d] = u[0] * a.binv[d] + u[1] * a.binv[3 + d] + u[2] * a.binv[6 + d];
        f[d] -= rint(f[d]);
      }
      for (int d = 0; d < 3; ++d) u[d] = f[0] * a.lat[d] + f[1] * a.lat[3 + d] + f[2] * a.lat[6 + d];
    }
    for (int d = 0; d < 3; ++d) d2 += u[d] * u[d];
    atomicMax(a.disp, (unsigned long long)__double_as_longlong(d2));
  }
}

int launch_filter(tm_system* s) {
  tm_ctx* ctx = s->ctx;
  const tm_consts& k = s->model->k;
  FiltArgs a;
  a.x = s->d_x; a.x0 = s->d_x_at_build; a.xhi = s->d_xhi; a.xlo = s->d_xlo;
  a.cand = s->d_cand; a.ccnt = s->d_ccnt; a.cnt_r = s->d_cnt_r; a.cnt_a = s->d_cnt_a;
  a.nbr_r = s->d_nbr_r; a.nbr_a = s->d_nbr_a; a.need = s->d_need; a.disp = s->d_disp;
  a.N = s->N; a.KC = s->KC; a.KR = s->KR; a.KA = s->KA; a.periodic = s->periodic ? 1 : 0;
  a.rr = k.r_rc_d; a.ra = k.a_rc_d;
  a.rr2_lo = (float)(k.r_rc_d * k.r_rc_d) * (1.f - kBand);
  a.rr2_hi = (float)(k.r_rc_d * k.r_rc_d) * (1.f + kBand);
  a.ra2_lo = (float)(k.a_rc_d * k.a_rc_d) * (1.f - kBand);
  a.ra2_hi = (float)(k.a_rc_d * k.a_rc_d) * (1.f + kBand);
  for (int q = 0; q < 9; ++q) {
    a.lat[q] = s->lat[q];
    a.binv[q] = s->binv[q];
  }
  a.ortho = s->ortho ? 1 : 0;
  tm_fill_shifts(s, a.sh_hi, a.sh_lo);
  k_nbr_filter<<<tm_div_up(s->N, 4), 128, 0, ctx->stream>>>(a);
  ctx->launches++;
  return tm_cuda_check(ctx, cudaGetLastError(), "filter");
}

}  // namespace

int tm_launch_positions(tm_system* s) {
  tm_ctx* ctx = s->ctx;
  k_positions<<<tm_div_up(s->N, 256), 256, 0, ctx->stream>>>(s->d_x, s->d_elem, s->d_xhi, s->d_xlo,
                                                             s->N, ctx->d_status);
  ctx->launches++;
  return tm_cuda_check(ctx, cudaGetLastError(), "positions");
}

// The Coulomb grid: about 24 atoms per cell, atoms packed in cell order, and
// the table of centre blocks. Enqueued on the ctx's second stream (which
// `ctx->stream` names while this runs); needs only positions and chunk boxes.
static int launch_ee_grid(tm_system* s) {
  tm_ctx* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  int rc;
  k_grid_from_chunks<<<tm_div_up(s->nmol, 4), 128, 0, st>>>(
      s->d_cbox, s->d_mol_chunk, s->d_off, s->d_egrid, s->d_encell_m, s->nmol, 2.0,
      s->periodic ? 1 : 0, s->hpl[0], s->hpl[1], s->hpl[2], 24.0, 0.125, 8.0, s->ee_dims[0],
      s->ee_dims[1], s->ee_dims[2], s->nmol == 1 ? s->d_encell : nullptr, s->ecell_cap,
      ctx->d_status);
  if (s->nmol > 1) {
    k_grid_offsets<<<1, 256, 0, st>>>(s->d_egrid, s->d_encell_m, s->nmol, s->d_encell, s->ecell_cap,
                                     ctx->d_status);
    ctx->launches++;
  }
  cudaMemsetAsync(s->d_ecell_cnt, 0, sizeof(int32_t) * (s->ecell_cap + 1), st);
  k_cell_count<<<tm_div_up(s->N, 256), 256, 0, st>>>(s->d_x, s->d_mol, s->d_egrid, s->d_ecell_cnt,
                                                      s->d_ecell_of_atom, s->N, s->ecell_cap,
                                                      ctx->d_status, tm_mat3_of(s->nrm));
  ctx->launches += 2;
  if ((rc = scan_exclusive<int32_t>(ctx, s->d_ecell_cnt, s->d_ecell_start, s->ecell_cap + 1,
                                    nullptr, s->d_scan_tmp2)))
    return rc;
  cudaMemsetAsync(s->d_ecell_cnt, 0, sizeof(int32_t) * (s->ecell_cap + 1), st);
  k_cell_fill<<<tm_div_up(s->N, 256), 256, 0, st>>>(s->d_ecell_of_atom, s->d_ecell_start,
                                                     s->d_ecell_cnt, s->d_ecell_atoms, s->N);
  k_cell_sort<<<tm_div_up(s->ecell_cap, 4), 128, 0, st>>>(s->d_ecell_start, s->d_ecell_atoms,
                                                            s->d_sort_tmp2, s->d_encell, s->ecell_cap);
  k_ee_pack<<<tm_div_up(s->N, 256), 256, 0, st>>>(s->d_ecell_atoms, s->d_x, s->d_elem, s->d_mol,
                                                  s->d_egrid, s->d_ecell_of_atom, s->d_epos,
                                                  s->d_exhi, s->N, tm_mat3_of(s->lat));
  cudaMemsetAsync(s->d_neblk, 0, sizeof(int32_t), st);
  k_ee_blocks<<<tm_div_up(s->N, 256), 256, 0, st>>>(s->d_ecell_atoms, s->d_mol, s->d_egrid,
                                                    s->d_ecell_of_atom, s->d_ecell_start,
                                                    s->d_eblk, s->d_neblk, s->N,
                                                    s->N / 32 + s->ecell_cap + 1, ctx->d_status);
  ctx->launches += 4;
  return tm_cuda_check(ctx, cudaGetLastError(), "coulomb grid");
}

// Bins atoms and builds both neighbour lists on the ctx stream without any
// host synchronisation. A centre with more neighbours than its row capacity
// records the count it needed in s->d_need; tm_nlist_grow() checks that after
// the caller's own sync point and enlarges the rows so the call can be redone.
static int launch_nbr_rows(tm_system* s);

int tm_launch_nlist(tm_system* s) {
  tm_ctx* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  int rc;
  if ((rc = tm_launch_positions(s))) return rc;
  k_cbox_chunks<<<s->nchunk, 256, 0, st>>>(s->d_chunk, s->d_xhi, s->d_cbox);
  ctx->launches++;
  // the Coulomb grid on the second stream, beside the neighbour rows; joined
  // on every path before this function returns
  cudaEventRecord(ctx->ev_fork, st);
  cudaStreamWaitEvent(ctx->aux, ctx->ev_fork, 0);
  ctx->stream = ctx->aux;
  rc = launch_ee_grid(s);
  ctx->stream = st;
  cudaEventRecord(ctx->ev_join, ctx->aux);
  if (!rc) rc = launch_nbr_rows(s);
  cudaStreamWaitEvent(st, ctx->ev_join, 0);
  if (rc) return rc;
  if (s->skin <= 0.0)
    cudaMemcpyAsync(s->d_x_at_build, s->d_x, sizeof(double) * 3 * s->N, cudaMemcpyDeviceToDevice, st);
  s->nlist_valid = true;
  return tm_cuda_check(ctx, cudaGetLastError(), "nlist");
}

// The neighbour grid and the exact rows (radial, angular; candidates when the
// system has a skin) with their reverse-edge indices, on the ctx stream.
static int launch_nbr_rows(tm_system* s) {
  tm_ctx* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  const tm_consts& k = s->model->k;
  int rc;
  k_grid_from_chunks<<<tm_div_up(s->nmol, 4), 128, 0, st>>>(
      s->d_cbox, s->d_mol_chunk, s->d_off, s->d_grid, s->d_ncell_m, s->nmol, k.r_rc_d + s->skin,
      s->periodic ? 1 : 0, s->hpl[0], s->hpl[1], s->hpl[2], 0.0, 2.0, 64.0, 0, 0, 0,
      s->nmol == 1 ? s->d_ncell : nullptr, s->ncell_cap, ctx->d_status);
  ctx->launches++;
  if (s->nmol > 1) {
    k_grid_offsets<<<1, 256, 0, st>>>(s->d_grid, s->d_ncell_m, s->nmol, s->d_ncell, s->ncell_cap,
                                     ctx->d_status);
    ctx->launches++;
  }
  cudaMemsetAsync(s->d_cell_cnt, 0, sizeof(int32_t) * (s->ncell_cap + 1), st);
  k_cell_count<<<tm_div_up(s->N, 256), 256, 0, st>>>(s->d_x, s->d_mol, s->d_grid, s->d_cell_cnt,
                                                      s->d_cell_of_atom, s->N, s->ncell_cap,
                                                      ctx->d_status, tm_mat3_of(s->nrm));
  ctx->launches++;
  if ((rc = scan_exclusive<int32_t>(ctx, s->d_cell_cnt, s->d_cell_start, s->ncell_cap + 1,
                                    nullptr, s->d_scan_tmp)))
    return rc;
  cudaMemsetAsync(s->d_cell_cnt, 0, sizeof(int32_t) * (s->ncell_cap + 1), st);
  k_cell_fill<<<tm_div_up(s->N, 256), 256, 0, st>>>(s->d_cell_of_atom, s->d_cell_start,
                                                     s->d_cell_cnt, s->d_cell_atoms, s->N);
  k_cell_sort<<<tm_div_up(s->ncell_cap, 4), 128, 0, st>>>(s->d_cell_start, s->d_cell_atoms,
                                                           s->d_sort_tmp, s->d_ncell, s->ncell_cap);
  ctx->launches += 2;
  if (!s->need_sticky) cudaMemsetAsync(s->d_need, 0, sizeof(int32_t) * 2, st);
  NbrArgs a = make_nbr_args(s, s->d_need);
  if (s->skin > 0.0) {
    // candidates: every neighbour within AN1_r_Rc + skin (FP64 test at that
    // radius), sorted as the rows are; the rows themselves come from the filter
    if (!s->need_sticky) cudaMemsetAsync(s->d_need_c, 0, sizeof(int32_t) * 2, st);
    a.need = s->d_need_c;
    a.nbr_r = s->d_cand;
    a.cnt_r = s->d_ccnt;
    a.KR = s->KC;
    a.KA = 1;              // no angular entries (ra = 0); the angular counts
                           // written here are replaced by the filter
    a.rr = k.r_rc_d + s->skin;
    a.rr2_lo = (float)(a.rr * a.rr) * (1.f - kBand);
    a.rr2_hi = (float)(a.rr * a.rr) * (1.f + kBand);
    a.ra = 0.0;
    a.ra2_lo = a.ra2_hi = -1.f;
  }
  const size_t shm = (size_t)4 * (a.KR + a.KA) * sizeof(uint64_t);
  if (shm > 48 * 1024) {
    cudaFuncSetAttribute(k_nbr_build<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
    cudaFuncSetAttribute(k_nbr_build<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  }
  if (s->periodic)
    k_nbr_build<true><<<tm_div_up(s->N, 4), 128, shm, st>>>(a);
  else
    k_nbr_build<false><<<tm_div_up(s->N, 4), 128, shm, st>>>(a);
  ctx->launches++;
  if (s->skin > 0.0) {
    cudaMemsetAsync(s->d_disp, 0, sizeof(unsigned long long), st);
    cudaMemcpyAsync(s->d_x_at_build, s->d_x, sizeof(double) * 3 * s->N, cudaMemcpyDeviceToDevice, st);
    if ((rc = launch_filter(s))) return rc;
    s->cand_valid = true;
    s->cand_rebuild = false;
  }
  k_nbr_reverse<<<tm_div_up(2 * s->N, 4), 128, 0, st>>>(s->d_nbr_r, s->d_cnt_r, s->d_rev_r, s->KR,
                                                        s->d_nbr_a, s->d_cnt_a, s->d_rev_a, s->KA,
                                                        s->d_elem, s->d_mol, s->d_off, s->N);
  ctx->launches += 1;
  return tm_cuda_check(ctx, cudaGetLastError(), "neighbour rows");
}

// Skin lists between candidate builds: positions, exact rows filtered from
// the candidates, reverse edges, and the Coulomb-grid packing of the current
// positions into the cells of the last build.
int tm_launch_nlist_filter(tm_system* s) {
  tm_ctx* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  int rc;
  if ((rc = tm_launch_positions(s))) return rc;
  if (!s->need_sticky) cudaMemsetAsync(s->d_need, 0, sizeof(int32_t) * 2, st);
  if ((rc = launch_filter(s))) return rc;
  k_nbr_reverse<<<tm_div_up(2 * s->N, 4), 128, 0, st>>>(s->d_nbr_r, s->d_cnt_r, s->d_rev_r, s->KR,
                                                        s->d_nbr_a, s->d_cnt_a, s->d_rev_a, s->KA,
                                                        s->d_elem, s->d_mol, s->d_off, s->N);
  k_ee_pack<<<tm_div_up(s->N, 256), 256, 0, st>>>(s->d_ecell_atoms, s->d_x, s->d_elem, s->d_mol,
                                                  s->d_egrid, s->d_ecell_of_atom, s->d_epos,
                                                  s->d_exhi, s->N, tm_mat3_of(s->lat));
  ctx->launches += 2;
  s->nlist_valid = true;
  return tm_cuda_check(ctx, cudaGetLastError(), "nlist filter");
}

// After a stream sync: if the last build overflowed a row, enlarge the rows
// (to the next multiple of 32 above what was needed) and report it.
int tm_nlist_grow(tm_system* s, bool* grew) {
  tm_ctx* ctx = s->ctx;
  *grew = false;
  int32_t h_need[2] = {0, 0};
  int rc;
  if ((rc = tm_cuda_check(ctx, cudaMemcpyAsync(h_need, s->d_need, sizeof(h_need), cudaMemcpyDeviceToHost, ctx->stream), "need")) ||
      (rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "need")))
    return rc;
  if (h_need[0] <= s->KR && h_need[1] <= s->KA) return TM_OK;
  const int KR = h_need[0] > s->KR ? ((h_need[0] + 31) / 32) * 32 : s->KR;
  const int KA = h_need[1] > s->KA ? ((h_need[1] + 31) / 32) * 32 : s->KA;
  tm_free(ctx, s->d_nbr_r, sizeof(uint32_t) * (size_t)s->N_cap * s->KR);
  tm_free(ctx, s->d_rev_r, sizeof(int32_t) * (size_t)s->N_cap * s->KR);
  tm_free(ctx, s->d_sr, sizeof(float) * (size_t)s->N_cap * s->KR);
  tm_free(ctx, s->d_nbr_a, sizeof(uint32_t) * (size_t)s->N_cap * s->KA);
  tm_free(ctx, s->d_rev_a, sizeof(int32_t) * (size_t)s->N_cap * s->KA);
  tm_free(ctx, s->d_va, sizeof(float4) * (size_t)s->N_cap * s->KA);
  s->bytes -= (sizeof(uint32_t) + sizeof(int32_t) + sizeof(float)) * (size_t)s->N_cap * s->KR +
              (sizeof(uint32_t) + sizeof(int32_t) + sizeof(float4)) * (size_t)s->N_cap * s->KA;
  s->KR = KR;
  s->KA = KA;
  if ((rc = tm_alloc(ctx, (void**)&s->d_nbr_r, sizeof(uint32_t) * (size_t)s->N_cap * KR)) ||
      (rc = tm_alloc(ctx, (void**)&s->d_rev_r, sizeof(int32_t) * (size_t)s->N_cap * KR)) ||
      (rc = tm_alloc(ctx, (void**)&s->d_sr, sizeof(float) * (size_t)s->N_cap * KR)) ||
      (rc = tm_alloc(ctx, (void**)&s->d_nbr_a, sizeof(uint32_t) * (size_t)s->N_cap * KA)) ||
      (rc = tm_alloc(ctx, (void**)&s->d_rev_a, sizeof(int32_t) * (size_t)s->N_cap * KA)) ||
      (rc = tm_alloc(ctx, (void**)&s->d_va, sizeof(float4) * (size_t)s->N_cap * KA)))
    return rc;
  s->bytes += (sizeof(uint32_t) + sizeof(int32_t) + sizeof(float)) * (size_t)s->N_cap * KR +
              (sizeof(uint32_t) + sizeof(int32_t) + sizeof(float4)) * (size_t)s->N_cap * KA;
  s->nlist_valid = false;
  *grew = true;
  return TM_OK;
}

int tm_count_nlist(tm_system* s, int64_t counts[4]) {
  tm_ctx* ctx = s->ctx;
  std::vector<int32_t> cr(s->N), ca(s->N);
  int rc;
  if ((rc = tm_cuda_check(ctx, cudaMemcpyAsync(cr.data(), s->d_cnt_r, sizeof(int32_t) * s->N, cudaMemcpyDeviceToHost, ctx->stream), "cnt")) ||
      (rc = tm_cuda_check(ctx, cudaMemcpyAsync(ca.data(), s->d_cnt_a, sizeof(int32_t) * s->N, cudaMemcpyDeviceToHost, ctx->stream), "cnt")) ||
      (rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "cnt")))
    return rc;
  int64_t P = 0, T = 0, mx = 0;
  for (int i = 0; i < s->N; ++i) {
    P += cr[i];
    T += (int64_t)ca[i] * (ca[i] - 1) / 2;
    mx = cr[i] > mx ? cr[i] : mx;
  }
  int64_t ee = 0;
  if ((rc = tm_count_ee(s, &ee))) return rc;
  counts[0] = P; counts[1] = T; counts[2] = ee; counts[3] = mx;
  return TM_OK;
}

int tm_launch_export_nlist(tm_system* s, int64_t* radp, int64_t* angt, int64_t* mil_j,
                           int64_t* mil_jk, int64_t P, int64_t T) {
  tm_ctx* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  int rc;
  int64_t *pr = nullptr, *pt = nullptr, *sr = nullptr, *stt = nullptr;
  const size_t nb = sizeof(int64_t) * (size_t)(s->N + 1);
  if ((rc = tm_alloc(ctx, (void**)&pr, nb)) || (rc = tm_alloc(ctx, (void**)&pt, nb)) ||
      (rc = tm_alloc(ctx, (void**)&sr, nb)) || (rc = tm_alloc(ctx, (void**)&stt, nb)))
    return rc;
  k_export_sizes<<<tm_div_up(s->N, 256), 256, 0, st>>>(s->d_cnt_r, s->d_cnt_a, sr, stt, s->N);
  ctx->launches++;
  if ((rc = scan_exclusive<int64_t>(ctx, sr, pr, s->N, nullptr)) ||
      (rc = scan_exclusive<int64_t>(ctx, stt, pt, s->N, nullptr)))
    return rc;
  ExportArgs a;
  a.nbr_r = s->d_nbr_r; a.nbr_a = s->d_nbr_a; a.cnt_r = s->d_cnt_r; a.cnt_a = s->d_cnt_a;
  a.elem = s->d_elem; a.mol = s->d_mol; a.off = s->d_off; a.pr = pr; a.pt = pt;
  a.radp = radp; a.milj = mil_j; a.angt = angt; a.miljk = mil_jk;
  a.N = s->N; a.KR = s->KR; a.KA = s->KA; a.nele = s->model->k.nele;
  a.nreal_stride = 0;
  for (int p = 0; p < TM_MAX_ELE; ++p)
    for (int q = 0; q < TM_MAX_ELE; ++q) a.elepair[p][q] = s->model->k.elepair[p][q];
  k_export_lists<<<tm_div_up(s->N, 4), 128, 0, st>>>(a);
  ctx->launches++;
  rc = tm_cuda_check(ctx, cudaStreamSynchronize(st), "export");
  tm_free(ctx, pr, nb); tm_free(ctx, pt, nb); tm_free(ctx, sr, nb); tm_free(ctx, stt, nb);
  (void)P; (void)T;
  return rc;
}

static EEArgs make_ee_args(tm_system* s) {
  const tm_consts& k = s->model->k;
  EEArgs a;
  a.x = s->d_x; a.xhi = s->d_xhi; a.xlo = s->d_xlo; a.mol = s->d_mol; a.grid = s->d_grid;
  a.cell_of = s->d_cell_of_atom; a.cell_start = s->d_cell_start; a.cell_atoms = s->d_cell_atoms;
  a.offs = nullptr; a.count = nullptr; a.out = nullptr; a.N = s->N; a.ree = k.ree_d;
  a.ree2_lo = (float)(k.ree_d * k.ree_d) * (1.f - kBand);
  a.ree2_hi = (float)(k.ree_d * k.ree_d) * (1.f + kBand);
  for (int q = 0; q < 9; ++q) a.lat[q] = s->lat[q];
  a.periodic = s->periodic ? 1 : 0;
  return a;
}

int tm_count_ee(tm_system* s, int64_t* npairs) {
  tm_ctx* ctx = s->ctx;
  int rc;
  int64_t *cnt = nullptr, *offs = nullptr, *tot = nullptr;
  const size_t nb = sizeof(int64_t) * (size_t)(s->N + 1);
  if ((rc = tm_alloc(ctx, (void**)&cnt, nb)) || (rc = tm_alloc(ctx, (void**)&offs, nb)) ||
      (rc = tm_alloc(ctx, (void**)&tot, sizeof(int64_t))))
    return rc;
  EEArgs a = make_ee_args(s);
  a.count = cnt;
  k_ee_pairs<false><<<tm_div_up(s->N, 4), 128, 0, ctx->stream>>>(a);
  ctx->launches++;
  if ((rc = scan_exclusive<int64_t>(ctx, cnt, offs, s->N, tot))) return rc;
  int64_t h = 0;
  if ((rc = tm_cuda_check(ctx, cudaMemcpyAsync(&h, tot, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream), "ee")) ||
      (rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "ee")))
    return rc;
  *npairs = h;
  tm_free(ctx, cnt, nb); tm_free(ctx, offs, nb); tm_free(ctx, tot, sizeof(int64_t));
  return TM_OK;
}

int tm_launch_export_ee(tm_system* s, int64_t* eep, int64_t cap) {
  tm_ctx* ctx = s->ctx;
  int rc;
  int64_t *cnt = nullptr, *offs = nullptr, *tot = nullptr;
  const size_t nb = sizeof(int64_t) * (size_t)(s->N + 1);
  if ((rc = tm_alloc(ctx, (void**)&cnt, nb)) || (rc = tm_alloc(ctx, (void**)&offs, nb)) ||
      (rc = tm_alloc(ctx, (void**)&tot, sizeof(int64_t))))
    return rc;
  EEArgs a = make_ee_args(s);
  a.count = cnt;
  k_ee_pairs<false><<<tm_div_up(s->N, 4), 128, 0, ctx->stream>>>(a);
  ctx->launches++;
  if ((rc = scan_exclusive<int64_t>(ctx, cnt, offs, s->N, tot))) return rc;
  int64_t h = 0;
  if ((rc = tm_cuda_check(ctx, cudaMemcpyAsync(&h, tot, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream), "ee")) ||
      (rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "ee")))
    return rc;
  if (h > cap) {
    tm_free(ctx, cnt, nb); tm_free(ctx, offs, nb); tm_free(ctx, tot, sizeof(int64_t));
    return tm_fail(ctx, TM_E_CAPACITY, "ee export buffer too small");
  }
  a.offs = offs;
  a.out = eep;
  k_ee_pairs<true><<<tm_div_up(s->N, 4), 128, 0, ctx->stream>>>(a);
  ctx->launches++;
  rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "ee fill");
  tm_free(ctx, cnt, nb); tm_free(ctx, offs, nb); tm_free(ctx, tot, sizeof(int64_t));
  return rc;
}

// ---------------------------------------------------------------------------
// Allocation-free neighbour-list build (tm_nlist_build_static)
//
// For callers that own every byte of device memory themselves and cannot let
// a library call cudaMalloc (a host MD engine or plugin that hands the GPU a
// fixed arena, a serving process whose memory is budgeted up front): the
// scratch of the cell-list build lives in one file-scope device array of fixed
// size, held on every GPU that loads this code until the process exits. Under
// CUDA's lazy module loading (the default) the array is committed when this
// file's module first loads on a device: at the first call of this entry
// point or the first neighbour-list build there. The device address is looked
// up once per device, in the context current at that first call (the device's
// primary context); it is not looked up again after cudaDeviceReset.
// ---------------------------------------------------------------------------
#define TM_STATIC_MAX_ATOMS 32768
#define TM_STATIC_MAX_CELLS (2 * TM_STATIC_MAX_ATOMS + 64)

namespace {

struct StaticScratch {
  float4 xhi[TM_STATIC_MAX_ATOMS];
  float4 xlo[TM_STATIC_MAX_ATOMS];
  int32_t mol[TM_STATIC_MAX_ATOMS];
  int32_t cell_atoms[TM_STATIC_MAX_ATOMS];
  int32_t cell_of_atom[TM_STATIC_MAX_ATOMS];
  int32_t sort_tmp[TM_STATIC_MAX_ATOMS];
  int32_t cell_cnt[TM_STATIC_MAX_CELLS + 1];
  int32_t cell_start[TM_STATIC_MAX_CELLS + 1];
  tm_grid grid;
  tm_dev_status status;
  int32_t off[2];
  int32_t ncell;
  int32_t ncell_m;
  int32_t need[2];
};

// Every call shares this array; it keeps the previous call's contents.
static __device__ __align__(256) StaticScratch g_static_scratch;

constexpr int kMaxDevices = 64;
StaticScratch* g_static_ptr[kMaxDevices] = {};

__global__ void k_static_init(StaticScratch* s, int N) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) s->mol[i] = 0;
  if (i == 0) {
    s->off[0] = 0;
    s->off[1] = N;
    s->need[0] = 0;
    s->need[1] = 0;
    s->status.code = 0;
    s->status.detail = 0;
    s->status.where = 0;
  }
}

// single-block exclusive scan of n <= 1024 * 80 ints (the cell counts)
__global__ void k_scan_single(const int32_t* __restrict__ in, int32_t* __restrict__ out, int n) {
  __shared__ int32_t part[1024];
  const int per = (n + 1023) / 1024;
  const int b = threadIdx.x * per;
  int32_t sum = 0;
  for (int q = 0; q < per; ++q)
    if (b + q < n) sum += in[b + q];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int32_t t = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += t;
    __syncthreads();
  }
  int32_t run = part[threadIdx.x] - sum;
  for (int q = 0; q < per; ++q)
    if (b + q < n) {
      out[b + q] = run;
      run += in[b + q];
    }
}

}  // namespace

extern "C" int tm_nlist_build_static(const double* x, const int32_t* elem, int natoms,
                                     double r_rc, double a_rc, int32_t* cnt_r, uint32_t* nbr_r,
                                     int KR, int32_t* cnt_a, uint32_t* nbr_a, int KA,
                                     int32_t needed[2], void* stream) {
  if (!x || !elem || !cnt_r || !nbr_r || !cnt_a || !nbr_a || natoms <= 0 || KR <= 0 || KA <= 0)
    return TM_E_ARG;
  if (natoms > TM_STATIC_MAX_ATOMS) return TM_E_ARG;          // beyond the fixed scratch
  if (!(a_rc > 0.0 && a_rc <= r_rc)) return TM_E_ARG;
  if ((size_t)4 * (KR + KA) * sizeof(uint64_t) > 200 * 1024) return TM_E_ARG;
  // an error left by the caller's earlier work is not this call's: clear it
  (void)cudaGetLastError();
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TM_E_CUDA;
  // first call on this device: resolve the device address of the scratch
  // (the host-side symbol is only a stand-in and must never reach a kernel)
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return TM_E_CUDA;
    g_static_ptr[dev] = static_cast<StaticScratch*>(p);
  }
  StaticScratch* S = g_static_ptr[dev];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the call copies counts to the host and synchronises the stream: neither
  // may happen inside a stream capture
  cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap_status) != cudaSuccess) return TM_E_CUDA;
  if (cap_status != cudaStreamCaptureStatusNone) return TM_E_ARG;
  const int N = natoms;
  const int cap = 2 * N + 64;
  k_static_init<<<tm_div_up(N, 256), 256, 0, st>>>(S, N);
  k_positions<<<tm_div_up(N, 256), 256, 0, st>>>(x, elem, S->xhi, S->xlo, N, &S->status);
  k_grid_setup<<<1, 256, 0, st>>>(x, S->off, &S->grid, &S->ncell_m, r_rc, 0, 0.0, 0.0, 0.0, 0.0,
                                  2.0, 64.0, 0, 0, 0);
  k_grid_offsets<<<1, 256, 0, st>>>(&S->grid, &S->ncell_m, 1, &S->ncell, cap, &S->status);
  if (cudaMemsetAsync(S->cell_cnt, 0, sizeof(int32_t) * (cap + 1), st) != cudaSuccess) return TM_E_CUDA;
  const double ident[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};   // open boundary: Cartesian bins
  k_cell_count<<<tm_div_up(N, 256), 256, 0, st>>>(x, S->mol, &S->grid, S->cell_cnt, S->cell_of_atom,
                                                   N, cap, &S->status, tm_mat3_of(ident));
  k_scan_single<<<1, 1024, 0, st>>>(S->cell_cnt, S->cell_start, cap + 1);
  if (cudaMemsetAsync(S->cell_cnt, 0, sizeof(int32_t) * (cap + 1), st) != cudaSuccess) return TM_E_CUDA;
  k_cell_fill<<<tm_div_up(N, 256), 256, 0, st>>>(S->cell_of_atom, S->cell_start, S->cell_cnt,
                                                  S->cell_atoms, N);
  k_cell_sort<<<tm_div_up(cap, 4), 128, 0, st>>>(S->cell_start, S->cell_atoms, S->sort_tmp, &S->ncell,
                                                 cap);
  NbrArgs a;
  a.x = x; a.xhi = S->xhi; a.xlo = S->xlo; a.mol = S->mol; a.elem = elem; a.grid = &S->grid;
  a.cell_of = S->cell_of_atom; a.cell_start = S->cell_start; a.cell_atoms = S->cell_atoms;
  a.cnt_r = cnt_r; a.cnt_a = cnt_a; a.nbr_r = nbr_r; a.nbr_a = nbr_a; a.need = S->need;
  a.N = N; a.KR = KR; a.KA = KA; a.rr = r_rc; a.ra = a_rc;
  a.rr2_lo = (float)(r_rc * r_rc) * (1.f - kBand);
  a.rr2_hi = (float)(r_rc * r_rc) * (1.f + kBand);
  a.ra2_lo = (float)(a_rc * a_rc) * (1.f - kBand);
  a.ra2_hi = (float)(a_rc * a_rc) * (1.f + kBand);
  for (int q = 0; q < 9; ++q) a.lat[q] = 0.0;
  const size_t shm = (size_t)4 * (KR + KA) * sizeof(uint64_t);
  if (shm > 48 * 1024 &&
      cudaFuncSetAttribute(k_nbr_build<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm) !=
          cudaSuccess)
    return TM_E_CUDA;
  k_nbr_build<false><<<tm_div_up(N, 4), 128, shm, st>>>(a);
  if (cudaGetLastError() != cudaSuccess) return TM_E_CUDA;
  // the counters the caller needs to size its rows, and the status word
  int32_t h[2] = {0, 0};
  tm_dev_status hs;
  if (cudaMemcpyAsync(h, S->need, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&hs, &S->status, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return TM_E_CUDA;
  if (needed) {
    needed[0] = h[0];
    needed[1] = h[1];
  }
  if (hs.code) return hs.code;
  if (h[0] > KR || h[1] > KA) return TM_E_CAPACITY;
  return TM_OK;
}
