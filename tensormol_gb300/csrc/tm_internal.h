// Internal host/device structures of libtmgpu (not part of the ABI).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/tmgpu.h"
#include "tm_common.cuh"

#define TM_MAX_ELE 8
#define TM_MAX_HIDDEN 4
#define TM_BN 256          // padding of the hidden width H and descriptor width Dp
#define TM_KINK_LAYERS 8   // entry counters of the relu refinement (one per forward layer)
#define TM_CHUNK 256      // atoms per reduction chunk (one block, one atom per thread)
#define TM_BM 128          // GEMM M tile (rows per element are padded to this)
#define TM_EE_SPLIT 25     // warps sharing one centre block's half stencil (one
                           // (x, y) column each at a 3-cell reach)

// Constants of the model read by the device kernels (passed by value).
struct tm_consts {
  int nele, nelep, nr, na_rs, na_as, D, Dp;
  int act;
  float alpha_sig;
  float r_rc, a_rc, eta, zeta, zeta_pow2;  // zeta_pow2: 1 when zeta == 8
  float pi_tf;                              // 3.14159265359 as in RawSymFunc.py
  float rs_r[32], rs_a[8], cos_th[8], sin_th[8];
  float two_1mz;                            // 2^(1 - zeta)
  // low parts of the constants above (value - fp32(value)) and the cutoff
  // functions' fc(r) = sin^2(c (Rc - r)), c = pi / (2 Rc), as hi + lo pairs:
  // the double-single descriptor arithmetic of the relu refinement
  float rs_r_lo[32], rs_a_lo[8], cos_th_lo[8], sin_th_lo[8];
  float r_rc_hi, r_rc_lo, a_rc_hi, a_rc_lo, cr_hi, cr_lo, ca_hi, ca_lo;
  int elepair[TM_MAX_ELE][TM_MAX_ELE];      // unordered element pair -> index
  // Coulomb / vdW (atomic units, see params.coulomb_constants)
  float bohr, alpha, r_lr, r_sr, elu_shift, elu_a, zz, yy;
  float vdw_width, vdw_begin;
  // erfc(x) = exp(-x^2) P(t) on the DSF range x = alpha r, r in [r_sr, r_lr]:
  // P interpolates erfcx at Chebyshev nodes, t = x erfc_s + erfc_o in [-1, 1];
  // erfc_n = 0: the range needs more than degree 10 (erfcf is used instead)
  float erfc_c[11], erfc_s, erfc_o;
  int erfc_n;
  float c6[TM_MAX_ELE], r0[TM_MAX_ELE];
  double r_rc_d, a_rc_d, ree_d;             // membership radii (FP64 test)
  float ree;
  int add_ecc, has_vdw;
};

// Per-molecule cell grid.
struct tm_grid {
  double ox, oy, oz;      // origin
  double cx, cy, cz;      // cell edge per dimension
  int nx, ny, nz;
  int cell_off;           // first global cell index
  int periodic;
  int atom_off, natom;    // atoms of the molecule
  int pad;
};

struct tm_ctx {
  int device = 0;
  int num_sms = 1;                     // streaming multiprocessors of the device
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // second stream of the library's own: the pair terms run on it beside the
  // network backward pass (forked from and joined back into `stream`)
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  size_t budget = 0, in_use = 0;
  int64_t launches = 0;
  tm_dev_status* d_status = nullptr;
  tm_dev_status* h_status = nullptr;   // pinned
  std::string err;
  PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
};

struct tm_layer_host {
  std::vector<double> W, b;
  int fan_in = 0, fan_out = 0;
  bool set = false;
};

struct tm_model {
  tm_ctx* ctx = nullptr;
  tm_model_desc desc;
  tm_consts k;
  int H = 0;         // padded hidden width (multiple of TM_BN), all layers equal
  int nlayer = 0;    // hidden layers
  bool final_ = false;
  // host copies: [net][ele][layer]
  std::vector<tm_layer_host> layers;  // index (net*nele + e)*(nlayer+1) + l
  // device weights (row-major, stacked over net, element):
  //   fwd[l]: W^T [2*nele*Nout_l][Kin_l] (hi, lo), bwd[l]: W [2*nele*Kin_l][Nout_l]
  void* w_fwd[TM_MAX_HIDDEN][2] = {};
  void* w_bwd[TM_MAX_HIDDEN][2] = {};
  float* bias[TM_MAX_HIDDEN] = {};     // [2][nele][H]
  float* wout = nullptr;               // [2][nele][H]  last layer weight vector
  double* bout = nullptr;              // [2][nele]
  CUtensorMap tm_wf[TM_MAX_HIDDEN][2];
  CUtensorMap tm_wb[TM_MAX_HIDDEN][2];
  // FP32 relu networks: the last hidden layer's backward weights with the
  // output weights folded in, W'[i][o] = W[i][o] w_out[o] (hi, lo); the
  // backward pass then starts from act'(z) in {0, 1}, one exact plane
  void* w_bwd_fold[2] = {};
  CUtensorMap tm_wbf[2];
  size_t elem_size = 4;                // 4 (tf32 split) or 2 (bf16)
  // relu refinement (FP32 precision with relu only): hidden pre-activations
  // within the tensor-core error bound of zero are recomputed in FP64
  bool kink = false;
  float2* kw2[TM_MAX_HIDDEN] = {};     // [2][nele][H][Kin_l] W^T as given (FP64) held as
                                       //   double-single pairs (hi, lo)
  float2* kb2[TM_MAX_HIDDEN] = {};     // [2][nele][H] biases, likewise
  float* kwn[TM_MAX_HIDDEN] = {};      // [2][nele][H] L2 norm of each W^T row (one output unit)
};

struct tm_system {
  tm_model* model = nullptr;
  tm_ctx* ctx = nullptr;
  int N = 0, nmol = 0;                 // current layout
  int N_cap = 0, nmol_cap = 0;         // allocated capacity (a layout may use less)
  int Mpad_cap = 0, nchunk_cap = 0, ncell_alloc = 0, ecell_alloc = 0;
  bool periodic = false;
  double lat[9] = {0};
  // general cells: unit normals of the three lattice planes (rows; plane d is
  // spanned by the other two lattice vectors, a_d . n_d > 0), their spacings,
  // and B^-1 (fractional f = x B^-1, f_d = sum_i x_i binv[3 i + d]); open
  // systems keep the identity normals, which bin by Cartesian coordinate
  double nrm[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  double hpl[3] = {0, 0, 0};
  double binv[9] = {0};
  bool ortho = true;                   // orthorhombic (or open)
  // a cell smaller than twice the largest cutoff across some plane spacing is
  // evaluated as a supercell of rep[0] x rep[1] x rep[2] copies (lat is then
  // the supercell's lattice, user_lat the cell's): the caller's N_user atoms
  // are copy 0, the others follow copy-major (atom a of copy c at c N_user + a)
  int rep[3] = {1, 1, 1};
  int K = 1;                           // number of copies
  int N_user = 0;
  double user_lat[9] = {0};
  double* d_xuser = nullptr;           // [N_user][3] caller positions (replicated systems)
  std::vector<int32_t> Z;              // host
  std::vector<int64_t> off;            // host
  std::vector<int32_t> elem_h;         // element index per atom
  // element-sorted MLP rows
  int Mpad = 0, ntiles = 0;
  std::vector<int32_t> row_of_atom_h, tile_elem_h;
  int32_t* row_of_atom = nullptr;
  int32_t* atom_of_row = nullptr;      // -1 for padding rows
  int32_t* tile_elem = nullptr;
  // atoms
  int32_t* d_Z = nullptr;
  int32_t* d_elem = nullptr;
  int32_t* d_mol = nullptr;            // molecule of atom
  int32_t* d_off = nullptr;            // [nmol+1]
  double* d_x = nullptr;               // [N][3]
  float4* d_xhi = nullptr;             // hi parts (w = element index)
  float4* d_xlo = nullptr;
  double* d_x_at_build = nullptr;      // positions at the last list build
  // cell grid
  tm_grid* d_grid = nullptr;           // [nmol]
  int ncell_cap = 0;
  int32_t* d_ncell = nullptr;          // total cells (device scalar)
  int32_t* d_ncell_m = nullptr;        // [nmol] cells per molecule
  int32_t* d_need = nullptr;           // [2] largest radial / angular count seen
  int32_t* d_cell_cnt = nullptr;       // [ncell_cap+1]
  int32_t* d_cell_start = nullptr;     // [ncell_cap+1]
  int32_t* d_cell_atoms = nullptr;     // [N]
  int32_t* d_cell_of_atom = nullptr;   // [N]
  int32_t* d_sort_tmp = nullptr;       // [N] scratch of the cell sort (crowded cells)
  int32_t* d_scan_tmp = nullptr;       // [4096] block sums of the cell-count scans
  int32_t* d_sort_tmp2 = nullptr;      // [N], [4096]: the same for the Coulomb grid, which
  int32_t* d_scan_tmp2 = nullptr;      //   is built on the second stream
  // coarser grid for the Coulomb/vdW pair terms (about 24 atoms per cell)
  int ee_dims[3] = {0, 0, 0};          // periodic: host-chosen cells per edge
  int ecell_cap = 0;
  tm_grid* d_egrid = nullptr;          // [nmol]
  int32_t* d_encell = nullptr;         // total cells (device scalar)
  int32_t* d_encell_m = nullptr;       // [nmol]
  int32_t* d_ecell_cnt = nullptr;      // [ecell_cap+1]
  int32_t* d_ecell_start = nullptr;    // [ecell_cap+1]
  int32_t* d_ecell_atoms = nullptr;    // [N] atoms in cell order
  int32_t* d_ecell_of_atom = nullptr;  // [N]
  int32_t* d_epos = nullptr;           // [N] position of an atom in cell order
  float4* d_exhi = nullptr;            // [N] cell-ordered hi parts (w = element)
  float4* d_exlo = nullptr;            // [N] cell-ordered lo parts (w = charge)
  unsigned long long* d_cacc = nullptr; // [5][N] pair-term fixed-point sums (cell order)
  void* h_stage = nullptr;             // pinned staging of the layout tables
  size_t h_stage_bytes = 0;
  cudaEvent_t stage_ev = nullptr;      // the staging buffer's copies are done
  int4* d_eblk = nullptr;              // [N/32 + ecell + 1] centre blocks: (column head cell,
                                       //   first atom, end atom) in cell order
  int32_t* d_neblk = nullptr;          // number of centre blocks (device scalar)
  // neighbour lists (ELL, per centre sorted by (element, reference index))
  int KR = 64, KA = 48;
  int32_t* d_cnt_r = nullptr;
  int32_t* d_cnt_a = nullptr;
  uint32_t* d_nbr_r = nullptr;         // [N*KR] packed (img << 27 | atom)
  uint32_t* d_nbr_a = nullptr;         // [N*KA]
  int32_t* d_rev_r = nullptr;          // [N*KR] j*KR + position of i in j's list
  int32_t* d_rev_a = nullptr;
  bool nlist_valid = false;
  bool need_sticky = false;            // keep the overflow counters across builds (MD chunks)
  // skin lists (MD): candidates within cutoff + skin, rebuilt when asked;
  // every step filters them with the exact membership rule
  double skin = 0.0;                   // 0: a full build every step
  bool cand_valid = false;
  bool cand_rebuild = true;            // the next build rebuilds the candidates
  int KC = 128;                        // candidate row capacity
  int32_t* d_ccnt = nullptr;           // [N] candidates per centre
  uint32_t* d_cand = nullptr;          // [N*KC] packed (img << 27 | atom), sorted like the rows
  int32_t* d_need_c = nullptr;         // [2] largest candidate count seen (on overflow)
  unsigned long long* d_disp = nullptr;  // squared displacement since the candidate build (bits)
  // descriptors + networks
  void* G[2] = {};                     // [Mpad][Dp] hi/lo (tf32) or bf16 (G[0])
  void* H1[2] = {};                    // [2*Mpad][H] per net stacked
  void* H2[2] = {};
  void* G3[2] = {};
  float* dEdG = nullptr;               // [2*Mpad][Dp]
  float* epart = nullptr;              // [2][Mpad][tm_gemm_row_parts(precision, H)]
  // relu refinement (tm_model::kink): squared row norms of each layer's input
  // (the bound of the tensor-core error), flags of the units to recompute and
  // the number recomputed by the last evaluation
  float* kink_g2 = nullptr;            // [Mpad] descriptor rows
  float* kink_h2[2] = {};              // [2][Mpad][row parts] partial sums, two
                                       //   buffers alternating between layers
  uint32_t* kink_mask = nullptr;       // [2][Mpad][H/32]
  uint32_t* kink_rows = nullptr;       // [2][Mpad][row parts] (row, part) entries with flags
  // relu networks: one bit per hidden unit, [z > 0], of each hidden layer
  // (written by the forward pass, read by the backward pass)
  uint32_t* relu_mask = nullptr;       // [TM_MAX_HIDDEN][2][Mpad][H/32]
  uint32_t* kink_nrows = nullptr;      // [TM_KINK_LAYERS] entries per forward layer
  unsigned long long* kink_count = nullptr;
  CUtensorMap tm_G[2], tm_H1[2], tm_H2[2], tm_G3[2];
  // 32-row boxes of the layer outputs for the GEMM epilogue's TMA stores (and
  // the backward pass's loads of the previous activation)
  CUtensorMap ts_H1[2], ts_H2[2], ts_G3[2], ts_dEdG;
  // per atom
  double* d_Eatom = nullptr;           // [N]
  float* d_qraw = nullptr;             // [N]
  float* d_q = nullptr;                // neutralised [N]
  float* d_dEdq = nullptr;             // [N]
  float4* d_fself = nullptr;           // [N] centre-side dE/dx from descriptors
  float* d_sr = nullptr;               // [N*KR] radial edge scalars
  float4* d_va = nullptr;              // [N*KA] angular edge vectors
  float4* d_fcv = nullptr;             // [N] Coulomb+vdW dE/dx (xyz), w unused
  double* d_ecv = nullptr;             // [N][2] per-atom half pair energies (cc, vdw)
  double* d_F = nullptr;               // [N][3] force (J/mol/A)
  double* d_mol_E = nullptr;           // [nmol][4]
  double* d_mol_aux = nullptr;         // [nmol][8]: sum q, sum dEdq~, dipole xyz
  // chunks of at most TM_CHUNK atoms of one molecule (two-level reductions)
  int nchunk = 0;
  int2* d_chunk = nullptr;             // [nchunk] (begin, end)
  int32_t* d_mol_chunk = nullptr;      // [nmol+1] first chunk of each molecule
  double* d_part = nullptr;            // [nchunk][8] partial sums
  float* d_cbox = nullptr;             // [nchunk][8] partial bounding boxes
  // export scratch
  int64_t* d_exp_off = nullptr;        // [N+1]
  size_t bytes = 0;
};

// ---- helpers (tm_api.cu) ----
int tm_fail(tm_ctx* ctx, int code, const std::string& msg);
int tm_cuda_check(tm_ctx* ctx, cudaError_t e, const char* what);
int tm_alloc(tm_ctx* ctx, void** p, size_t bytes);
void tm_free(tm_ctx* ctx, void* p, size_t bytes);
int tm_sync_status(tm_ctx* ctx, const char* what);
int tm_system_create_capacity(tm_model* m, int N_cap, int nmol_cap, tm_system** out);
int tm_system_relayout(tm_system* s, int N, int nmol, const int32_t* Z, const int64_t* off);
int tm_energy_force_device(tm_system* s, unsigned flags);

// ---- launchers ----
// tm_nlist.cu
int tm_launch_positions(tm_system* s);
int tm_launch_nlist(tm_system* s);
int tm_launch_nlist_filter(tm_system* s);   // skin lists: filter the candidates
int tm_nlist_grow(tm_system* s, bool* grew);
int tm_launch_export_nlist(tm_system* s, int64_t* radp, int64_t* angt, int64_t* mil_j,
                           int64_t* mil_jk, int64_t P, int64_t T);
int tm_count_ee(tm_system* s, int64_t* npairs);
int tm_launch_export_ee(tm_system* s, int64_t* eep, int64_t cap);
int tm_count_nlist(tm_system* s, int64_t counts[4]);
// tm_desc.cu
int tm_launch_descriptors(tm_system* s);
int tm_launch_adjoint(tm_system* s, unsigned flags);
// tm_gemm.cu
int tm_make_tmap(tm_ctx* ctx, CUtensorMap* map, void* base, int elem_bytes, uint64_t rows,
                 uint64_t cols, uint32_t box_rows);
int tm_launch_mlp(tm_system* s, bool backward);
int tm_launch_mlp_backward_only(tm_system* s);
int tm_profile_layers(tm_system* s, float* ms);   // [2 * nlayer] ms
int tm_gemm_bn(int prec);   // GEMM N tile of a precision mode (128 or 256)
int tm_gemm_row_parts(int prec, int H);   // partial sums per row of one layer launch
float tm_kink_kappa(int K); // relu refinement: flag bound per unit of ||a|| ||w||
int tm_gemm_selftest(tm_ctx* ctx, int prec, int M, int N, int K, const float* A,
                     const float* B, float* C, long long wait_limit = 0, int skip_it = -1);
// tm_coulomb.cu
int tm_launch_mlp_finish(tm_system* s);
int tm_launch_coulomb(tm_system* s, unsigned flags);
int tm_launch_finish(tm_system* s, unsigned flags);

static inline int tm_div_up(int a, int b) { return (a + b - 1) / b; }

// Nine doubles by value (a lattice, its inverse, or plane normals) for kernels.
struct tm_mat3 {
  double v[9];
};
static inline tm_mat3 tm_mat3_of(const double* p) {
  tm_mat3 m;
  for (int q = 0; q < 9; ++q) m.v[q] = p[q];
  return m;
}
