/*
 * tmgpu.h - C ABI of the GB300 (sm_103a) BP+EE energy-and-force library.
 *
 * This is the drop-in boundary for TensorMol's energy/force hot path: the
 * neighbour lists, ANI-1 descriptors, per-element BP energy and charge
 * networks, DSF/elu Coulomb + C6 vdW between the network charges, forces,
 * and the integrators that consume them. Plain C types only: host or device
 * pointers and sizes, int status returns, no exceptions across the ABI.
 *
 * Units at the boundary are the reference's: positions in Angstrom, energies
 * in Hartree, forces in J mol^-1 A^-1 (TFNetworks/TFMolManage.py:1439),
 * velocities in A/fs and masses in kg/mol (Simulations/SimpleMD.py:14-51).
 *
 * Threading: one tm_ctx per host thread; calls on one ctx are not re-entrant.
 */
#ifndef TMGPU_H
#define TMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (every entry point returns one) ---------------------- */
#define TM_OK 0
#define TM_E_ARG 1          /* invalid argument or unsupported shape        */
#define TM_E_CUDA 2         /* CUDA runtime/driver error                    */
#define TM_E_CAPACITY 3     /* neighbour capacity exceeded (retry larger)   */
#define TM_E_NONFINITE 4    /* non-finite positions or outputs              */
#define TM_E_BUDGET 5       /* allocation would exceed the ctx HBM budget   */
#define TM_E_TIMEOUT 6      /* a bounded device wait gave up                */
#define TM_E_STATE 7        /* call out of order (e.g. weights not final)   */
#define TM_E_UNSUPPORTED 8  /* feature not available in this build          */

/* ---- enums ------------------------------------------------------------- */
/* Activations of Instance.AssignActivation (TFNetworks/TFInstance.py:108-140) */
#define TM_ACT_RELU 0
#define TM_ACT_SIGMOID_WITH_PARAM 1 /* log(1+exp(a x))/a, Util.py:200-201 */
#define TM_ACT_SOFTPLUS 2
#define TM_ACT_TANH 3
#define TM_ACT_ELU 4

/* Arithmetic of the network GEMMs (descriptors, Coulomb and adjoint are FP32) */
#define TM_PREC_FP32 0   /* 3-pass split TF32 on tcgen05, FP32 accumulate      */
#define TM_PREC_BF16 1   /* 1-pass BF16 on tcgen05, FP32 accumulate            */

/* tm_energy_force flags */
#define TM_F_ENERGY_ONLY 1u   /* DoForce=False (samples/test_tensormol01.py:61-69) */
#define TM_F_DEVICE_IO 2u     /* x/outputs are device pointers on the ctx stream */
#define TM_F_REUSE_NLIST 4u   /* keep the current lists (caller rebuilt them)    */
#define TM_F_REFERENCE_PERIODIC_FORCE 8u /* periodic: drop image-side terms as
                                            the reference's gradient does      */

/* MD integrator kinds (Simulations/SimpleMD.py) */
#define TM_MD_NVE 0        /* VelocityVerletStep, SimpleMD.py:14-38          */
#define TM_MD_NOSE 1       /* NoseThermostat.step, SimpleMD.py:104-129       */
#define TM_MD_NHC 2        /* Nose-Hoover chain, Martyna et al. 1996 (see docs) */

typedef struct tm_ctx tm_ctx;
typedef struct tm_model tm_model;
typedef struct tm_system tm_system;
typedef struct tm_md tm_md;
typedef struct tm_serve tm_serve;

/*
 * Model description. Mirrors MolInstance_DirectBP_EE_SymFunction's
 * constructor and SetANI1Param (TFNetworks/TFBehlerParinelloSymEE.py:660-777)
 * reading PARAMS (TMParams.py:26-37, 57-79, 140-154).
 */
typedef struct tm_model_desc {
  int n_elements;          /* sorted atomic numbers in elements[]            */
  int elements[8];
  int n_hidden;            /* HiddenLayers, e.g. {512, 512, 512}             */
  int hidden[4];
  int activation;          /* TM_ACT_*                                       */
  double sigmoid_alpha;    /* PARAMS["sigmoid_alpha"]                        */
  double r_rc, a_rc;       /* AN1_r_Rc, AN1_a_Rc                             */
  double eta, zeta;        /* AN1_eta, AN1_zeta                              */
  int n_r_rs, n_a_rs, n_a_as; /* AN1_num_r_Rs, AN1_num_a_Rs, AN1_num_a_As    */
  double ee_cut_on;        /* EECutoffOn (must be 0, as the reference asserts) */
  double ee_cut_off;       /* EECutoffOff                                    */
  double elu_width;        /* Elu_Width                                      */
  double dsf_alpha;        /* DSFAlpha                                       */
  double poly_width;       /* Poly_Width                                     */
  int add_ecc;             /* AddEcc                                         */
  int has_vdw;             /* HasVdw argument of EvalBPDirectEE*             */
  int precision;           /* TM_PREC_*                                      */
} tm_model_desc;

/* ---- context ----------------------------------------------------------- */
/* hbm_budget_bytes = 0 means no limit beyond the device. */
int tm_ctx_create(int device, size_t hbm_budget_bytes, tm_ctx **out);
int tm_ctx_destroy(tm_ctx *ctx);
/* Use a caller-owned cudaStream_t (NULL = the ctx's own stream). */
int tm_ctx_set_stream(tm_ctx *ctx, void *cuda_stream);
void *tm_ctx_stream(tm_ctx *ctx);
/* Last error message (after any non-zero return). */
int tm_ctx_last_error(tm_ctx *ctx, char *buf, int len);
size_t tm_ctx_bytes_in_use(tm_ctx *ctx);
/* Kernels launched by this ctx since creation (a counter kept on the host). */
int64_t tm_ctx_launch_count(tm_ctx *ctx);

/* ---- model ------------------------------------------------------------- */
/* Replaces MolInstance_DirectBP_EE_SymFunction.__init__ + EvalPrepare
 * (TFBehlerParinelloSymEE.py:660-736, 1452-1501). */
int tm_model_create(tm_ctx *ctx, const tm_model_desc *desc, tm_model **out);
/*
 * One dense layer of one element's network: W[fan_in][fan_out] row-major and
 * b[fan_out] (the reference's tf.matmul(inputs, weights) + biases orientation,
 * TFBehlerParinelloSymEE.py:914-929 for net 0 = EnergyNet, :975-996 for
 * net 1 = DipoleNet). layer = 0..n_hidden (the last is the 1-wide output).
 */
int tm_model_set_layer(tm_model *m, int net, int element_index, int layer,
                       const double *W, const double *b, int fan_in, int fan_out);
int tm_model_finalize(tm_model *m);
int tm_model_descriptor_width(const tm_model *m);
int tm_model_destroy(tm_model *m);

/* ---- system (atoms, molecules, cell, device-resident state) ------------ */
/*
 * A batch of molecules in CSR order: atoms of molecule m are
 * mol_offsets[m] .. mol_offsets[m+1]-1. Replaces the padded
 * [nmol, MaxNAtoms] feed of EvalBPDirectEEUpdateSet (TFMolManage.py:1260-1276).
 * cell: NULL for open boundaries, else 9 doubles of lattice vectors (rows,
 * any shape, Periodic.py:12-24); positions are expected inside the cell
 * (ModuloLattice, Periodic.py:87-100). When a plane spacing of the cell
 * (volume / area of the opposite faces) is below twice the largest cutoff,
 * several images of an atom reach another (the reference tessellates more
 * shells, Periodic.py:143-147): such a cell is evaluated as the smallest
 * supercell (at most 4096 copies) whose spacings reach twice the cutoff, and
 * tm_energy_force returns the energy per cell and the cell's own atoms'
 * forces, charges and per-atom energies; list export, the images-fixed force
 * (TM_F_REFERENCE_PERIODIC_FORCE) and MD of such a cell return
 * TM_E_UNSUPPORTED. Linearly dependent lattice vectors give TM_E_ARG.
 * Z is host memory.
 */
int tm_system_create(tm_model *m, int natoms, int nmol, const int32_t *Z,
                     const int64_t *mol_offsets, const double *cell, tm_system **out);
int tm_system_destroy(tm_system *s);
int tm_system_natoms(const tm_system *s);
/* Positions [natoms][3] in Angstrom; device pointer if on_device. */
int tm_system_set_positions(tm_system *s, const double *x, int on_device);
int tm_system_get_positions(tm_system *s, double *x, int on_device);

/*
 * Builds the radial (r < AN1_r_Rc, both directions) and angular (r < AN1_a_Rc)
 * neighbour lists from the current positions with the reference's FP64
 * membership test. Replaces NeighborListSet.buildPairsAndTriplesWithEleIndex-
 * Linear/Periodic (ForceModifiers/Neighbors.py:344-470) and MolEmb.Make_NList-
 * Naive (C_API/MolEmb.cpp:1180-1251).
 */
int tm_system_build_nlist(tm_system *s);
/* counts[0] = radial pairs P, [1] = triples T, [2] = Coulomb pairs (i<j,
 * r < EECutoffOff; periodic: both directions as the reference lists them),
 * [3] = max radial neighbours of one atom. */
int tm_system_nlist_counts(tm_system *s, int64_t counts[4]);
/*
 * Exports the lists in the reference's layout and sorted order:
 * radp[P][4] = (mol, i, j, l), angt[T][5] = (mol, i, j, k, l),
 * mil_j[P][4], mil_jk[T][4] = (mol, i, l, slot) (Neighbors.py:344-467),
 * eep[Pee][3] = (mol, i, j) (TFMolManage.py:1430-1431; periodic:
 * (mol, i, j) with j an index into the 27-image tessellation,
 * Periodic.py:131-181). Atom indices are molecule-local. Any pointer may be
 * NULL. Host int64 buffers unless on_device.
 */
int tm_system_export_nlist(tm_system *s, int64_t *radp, int64_t *angt, int64_t *mil_j,
                           int64_t *mil_jk, int on_device);
int tm_system_export_ee(tm_system *s, int64_t *eep, int64_t cap, int on_device);

/*
 * Energy and forces: EvalBPDirectEELinearSingle / EvalBPDirectEEUpdateSet /
 * EvalBPDirectEEUpdateSinglePeriodic (TFMolManage.py:1260-1358, 1410-1439).
 * x: positions [natoms][3] (NULL = use the resident ones).
 * E_out[nmol][4] = (Etotal, Ebp, Ecc, Evdw) in Hartree.
 * F_out[natoms][3] in J/mol/A (ignored with TM_F_ENERGY_ONLY).
 * q_out[natoms] neutralised charges, dipole_out[nmol][3] (bohr * e), may be NULL.
 * Eatom_out[natoms] per-atom network energies (Ebp_atom), may be NULL.
 */
int tm_energy_force(tm_system *s, const double *x, unsigned flags, double *E_out,
                    double *F_out, double *q_out, double *dipole_out, double *Eatom_out);

/* ---- molecular dynamics (device-resident FP64 state) ------------------- */
/*
 * kind: TM_MD_NVE / TM_MD_NOSE / TM_MD_NHC. dt in fs, T in K, chain = NHC
 * length. Masses come from Z (PhysicalData.ATOMICMASSES). The first
 * acceleration is zero, as VelocityVerlet.__init__ sets it (SimpleMD.py:359).
 */
int tm_md_create(tm_system *s, int kind, double dt_fs, double T_kelvin, int chain,
                 tm_md **out);
int tm_md_destroy(tm_md *md);
int tm_md_set_velocities(tm_md *md, const double *v, int on_device);
int tm_md_get_velocities(tm_md *md, double *v, int on_device);
/*
 * nsteps integrator steps, each with one energy+force evaluation on exact
 * neighbour rows (the reference builds its lists on every call,
 * TFMolManage.py:1418-1431). skin = 0: a full build every step. skin > 0 (A):
 * candidates within the cutoffs + skin are built when atoms may have moved
 * skin/2 (checked on the device, chunks replayed if exceeded) and filtered to
 * the exact rows every step; periodic positions are wrapped into the cell at
 * candidate builds and at the end. log[nsteps][4] (host, may be NULL) =
 * (potential Hartree, kinetic J/mol per atom, conserved J/mol, T_eff K).
 */
int tm_md_run(tm_md *md, int nsteps, double skin, double *log);

/* ---- serving: continuous batching of requests -------------------------- */
/*
 * No single counterpart in the reference: its drivers call EnergyAndForce
 * once per molecule and step (samples/test_tensormol01.py:61-69,
 * SimpleMD.py:391-424). A tm_serve holds up to max_atoms atoms in up to
 * max_mols molecules (one molecule per request in flight, device memory
 * allocated once, against the context's HBM budget) and advances all of them
 * with one fused energy+force evaluation per step.
 */
#define TM_SERVE_EF 0   /* energy + force at fixed positions          */
#define TM_SERVE_MD 1   /* velocity-Verlet step (SimpleMD.py:14-38)   */
#define TM_SERVE_OPT 2  /* one FIRE relaxation step (Bitzek et al. 2006) */
int tm_serve_create(tm_model *m, int max_atoms, int max_mols, double dt_fs, tm_serve **out);
int tm_serve_destroy(tm_serve *sv);
int tm_serve_info(const tm_serve *sv, int *max_atoms, int *max_mols, int *natoms, int *nmol,
                  size_t *bytes);
/*
 * New batch composition: nmol molecules (Z, offsets as tm_system_create,
 * mode[nmol] = TM_SERVE_*). src[natoms] gives, per atom of the new layout, its
 * index in the previous layout (its positions, velocities and accelerations
 * are kept on the device) or -(k+1) for the k-th new atom, whose position and
 * velocity are x_new[k], v_new[k] (host, packed) and whose acceleration starts
 * at zero (SimpleMD.py:359). nmol = 0 empties the batch. TM_E_CAPACITY when
 * the layout does not fit.
 */
int tm_serve_layout(tm_serve *sv, int nmol, const int32_t *Z, const int64_t *offsets,
                    const int32_t *mode, const int32_t *src, const double *x_new,
                    const double *v_new);
/*
 * One step of every molecule; E_out[nmol][4] (host, may be NULL) as
 * tm_energy_force; fmax_out[nmol] (host, may be NULL): the largest atomic
 * force (J/mol/A) of each TM_SERVE_OPT molecule (0 for the others), for the
 * caller's convergence test.
 */
int tm_serve_step(tm_serve *sv, double *E_out, double *fmax_out);
/* Positions, velocities, forces (J/mol/A) of molecule mol to host (each may be NULL). */
int tm_serve_read(tm_serve *sv, int mol, double *x, double *v, double *F);

/* ---- allocation-free entry point ---------------------------------------- */
/*
 * No counterpart in the reference. The radial/angular neighbour-list build of
 * tm_system_build_nlist for ONE open-boundary molecule, for callers that cannot
 * let a library call cudaMalloc: a host MD engine or plugin that owns a fixed
 * device arena, or a serving process whose memory is budgeted up front. It
 * allocates nothing (no cudaMalloc/cudaFree, no allocating library routine);
 * its scratch is one file-scope device array sized for at most 32768 atoms
 * (about 2 MB, held on every GPU that loads it until exit). With CUDA's lazy
 * module loading (the default) that memory is committed by the first call of
 * this entry point on each device, or by the first neighbour-list build
 * there: make one small call before sizing a fixed arena from the free
 * memory. The scratch's device address is looked up once per device, in the
 * context current at that first call (the primary context); do not use this
 * entry point after cudaDeviceReset in the same process.
 *
 * All array arguments are device pointers the caller allocated: x[natoms][3]
 * (Angstrom, FP64), elem[natoms] (element index, 0-based, sorted by Z as in the
 * model), outputs cnt_r[natoms], nbr_r[natoms][KR], cnt_a[natoms],
 * nbr_a[natoms][KA] in the library's row layout (per centre sorted by
 * (element, index); the low 27 bits of an entry are the neighbour's atom index,
 * the high bits the image code 13 of an open system). needed (host, may be NULL)
 * receives the largest radial and angular counts when a row overflowed, else
 * zeros. Returns TM_E_ARG for natoms > 32768, TM_E_CAPACITY when a row
 * overflowed (then retry with KR/KA >= needed). Runs on `stream` and
 * synchronises it before returning.
 * Every call copies counts to the host and synchronises `stream`, so it is
 * never made on a capturing stream (TM_E_ARG). Every call reuses the same
 * scratch (it clears what must start at zero); calls that overlap on the GPU
 * race.
 */
int tm_nlist_build_static(const double *x, const int32_t *elem, int natoms, double r_rc,
                          double a_rc, int32_t *cnt_r, uint32_t *nbr_r, int KR, int32_t *cnt_a,
                          uint32_t *nbr_a, int KA, int32_t needed[2], void *stream);

/* ---- diagnostics (used by the test-suite) ------------------------------ */
/*
 * Runs the tensor-core layer kernel alone: C[M][N] = A[M][K] . B[N][K]^T on
 * host FP32 arrays, in the given precision. M % 128 == 0, N % 256 == 0,
 * K % 64 == 0. No counterpart in the reference (it has no GPU kernels).
 */
int tm_selftest_gemm(tm_ctx *ctx, int precision, int M, int N, int K, const float *A,
                     const float *B, float *C);
/*
 * Exercises the bounded waits of the tensor-core layer kernel: a 256 x 256 x 256
 * selftest product in which the operand loads of one pipeline stage are never
 * issued (nothing faults: the copy does not exist) and every wait is limited to
 * wait_cycles SM cycles (1 .. 2^28). Returns TM_E_TIMEOUT when the waits ran out
 * as designed: the kernel has then freed its tensor memory and returned, and the
 * context (its status word cleared) runs the next call normally. No counterpart
 * in the reference (it has no GPU kernels).
 */
int tm_selftest_gemm_timeout(tm_ctx *ctx, int precision, int64_t wait_cycles);
/*
 * The polynomial the pair kernel evaluates erfc with on this model's DSF range
 * (erfc(x) = exp(-x^2) P(t), t = x * scale + offset in [-1, 1], x = alpha r
 * for r from the elu width to the Coulomb cutoff, in bohr): coeffs[11]
 * (monomials in t, degree *n; *n = 0 when erfcf is used instead) and the
 * range [*x0, *x1]. No counterpart in the reference (it calls tf.math.erfc).
 */
int tm_model_erfc_poly(const tm_model *m, float *coeffs, int *n, float *scale, float *offset,
                       double *x0, double *x1);
/*
 * Descriptor rows of every atom in atom order, FP32 [natoms][D], for the
 * current positions (lists are built if needed). Replaces reading
 * TFSymSet_Scattered_Linear_WithEle_Release's SymList (RawSymFunc.py:2267-2309).
 */
int tm_system_descriptors(tm_system *s, float *G_out);
/*
 * The outputs of hidden layer `layer` (0 .. n_hidden-1) of both networks from
 * the last evaluation, out[2][natoms][hidden[layer]] (net 0 = energy, 1 =
 * charge; atoms in input order): the activations h = act(z) of a hidden layer
 * before the last, and w_out * act'(z) (the backward pass's seed) for the last
 * one; for relu networks in FP32 mode the last one is act'(z) in {0, 1} (the
 * output weights are folded into the backward pass's first weights). Valid after an evaluation with TM_F_ENERGY_ONLY (the backward pass
 * reuses these buffers). No counterpart in the reference (TensorFlow keeps
 * its intermediate tensors internal).
 */
int tm_system_layer_outputs(tm_system *s, int layer, float *out);
/*
 * The network layers of the last evaluation run again (forward, then backward,
 * from the same descriptor rows) with CUDA events around each tensor-core
 * layer launch only: ms[2 * n_hidden] = forward layers 0 .. n_hidden-1, then
 * backward layers n_hidden-1 .. 0, in ms. No counterpart in the reference.
 */
int tm_system_profile_layers(tm_system *s, float *ms);
/*
 * FP32 mode with relu: the number of hidden-unit pre-activations that the
 * last evaluation recomputed in FP64 because they lay within the tensor-core
 * error bound of the kink (0 in other modes). No counterpart in the reference
 * (its FP64 TensorFlow graph has no such step).
 */
int tm_system_refined_units(tm_system *s, int64_t *n);
/*
 * One energy(+force) evaluation of the resident positions with CUDA events on
 * the ctx stream between stages; stage_ms[7] = (lists, descriptors, network
 * forward, network backward, pair terms, adjoint + force gather, total) in ms.
 * Every stage runs alone here, in this order on the ctx stream (an ordinary
 * evaluation overlaps the pair terms with the network backward pass and the
 * Coulomb grid with the neighbour rows on a second stream).
 * No counterpart in the reference (its TFMolManage timing is wall-clock).
 */
int tm_energy_force_profile(tm_system *s, unsigned flags, float *stage_ms);

#ifdef __cplusplus
}
#endif
#endif /* TMGPU_H */
