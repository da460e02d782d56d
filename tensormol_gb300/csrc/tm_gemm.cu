// Per-element BP network layers as tcgen05 tensor-core GEMMs (sm_103a).
//
// One launch computes one layer for every element and both networks
// (net 0: EnergyNet, 1: DipoleNet; TFBehlerParinelloSymEE.py:884-944,
// 946-1015): C[128 x BN tile] = A[rows of one element, K] . W^T, with the
// element of each 128-row tile taken from a table (rows of each element are
// padded to 128, so no tile mixes elements).
//
// Persistent CTAs (one per SM) walk the tiles:
//   warp EW      TMA producer: K-slices of A and B into a ring of 128-byte-
//                swizzled shared-memory stages (cp.async.bulk.tensor, mbarriers)
//   warp EW + 1  MMA issuer: one elected thread issues tcgen05.mma into FP32
//                accumulators in tensor memory (two tile buffers)
//   warps 0..EW-1  epilogue (EW = 8, two per tensor-memory lane quarter; 4 for
//                the FP32 backward pass of a smooth activation): tcgen05.ld 32
//                columns at a time, fused bias + activation (forward) or
//                activation-derivative product (backward), staged in shared
//                memory, bulk tensor stores.
// Precision modes:
//   TM_PREC_FP32  kind::tf32 with operands split as x = hi + lo (both rounded
//                 to nearest TF32, tm_tf32_split); BN = 128. The large term
//                 Ahi Bhi and the two small terms Ahi Blo + Alo Bhi go to
//                 separate accumulators that the epilogue adds: the tensor
//                 core's accumulation drops low-order bits at every
//                 instruction (measured: a bias toward zero growing with K),
//                 and keeping the correction terms out of the large
//                 accumulator removes two thirds of those roundings.
//   TM_PREC_BF16  kind::f16 with BF16 operands, one pass, FP32 accumulate;
//                 BN = 256.
// All waits on mbarriers are bounded (2^28 cycles, about 0.13 s); a timeout
// sets the device status word to TM_E_TIMEOUT and the CTA still frees its
// tensor memory; a launch that finds the status word already set returns at
// once.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "tm_internal.h"

namespace {

constexpr int BM = TM_BM;
constexpr int EPI_FWD = 0, EPI_FWD_LAST = 1, EPI_BWD = 2, EPI_OUT = 3;

struct GemmArgs {
  CUtensorMap a0, a1, b0, b1;
  CUtensorMap o0, o1;  // 32-row boxes of the outputs (FP32: 32 columns, hi and lo;
                       // BF16: 64 columns in o0; dE/dG: 32 FP32 columns in o0);
                       // the backward pass also loads the previous activation by them
  int K;             // reduction length
  int N;             // output width of one (net, element) block
  int a_net_rows;    // row offset of net 1 in A (0 when both nets read the same A)
  int nele;
  const int32_t* tile_elem;
  int Mpad;
  int act;
  float alpha;
  const float* bias;   // [2][nele][N]
  const float* wout;   // [2][nele][N]
  float* epart;        // [2][Mpad][2 N/BN]: per (N tile, column half), BN of the precision mode
  void* out0;
  void* out1;
  int ldo;
  // relu: the backward pass takes act'(z) = [z > 0] from one bit per unit that
  // the forward pass of the layer wrote (and the refinement corrected), not
  // from the stored activation
  uint32_t* rmask_out;      // [2][Mpad][N/32] (forward, hidden layers), or null
  const uint32_t* rmask_in; // [2][Mpad][N/32] (backward), or null
  const void* hprev0;
  const void* hprev1;
  tm_dev_status* st;
  int mtiles, ntiles;   // tiles per net along M and N
  // relu refinement (FP32 forward layers with relu): a unit is flagged when
  // |z| < kappa ||a_row|| ||w_unit||, a bound of the tensor-core error
  const float* an2;     // squared norms of the input rows: an2_parts partial sums per row
  int an2_parts;
  int an2_net_stride;   // floats between the two nets' rows (0: shared input)
  float* hn2_out;       // [2][Mpad][2 ntiles] partial squared norms of the outputs (or null)
  const float* wnorm;   // [2][nele][N]
  uint32_t* kmask;      // [2][Mpad][N/32]
  uint32_t* krows;      // entries orow * parts + part with a flagged unit, appended
  uint32_t* knrows;     // number of entries (zeroed before the launch)
  float kappa;
  // diagnostics of the bounded waits (tm_selftest_gemm_timeout): the wait
  // limit in SM cycles (0: 2^28) and a producer iteration whose operand
  // loads are withheld (-1: none), so that the MMA issuer's wait runs out
  long long wait_limit;
  int skip_it;
  // A has no lo part (FP32: the relu seed act'(z) in {0, 1}, exact in TF32):
  // its lo loads and the A_lo B_hi instruction are skipped
  int a_single;
};

// ---- PTX wrappers ---------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t cnt) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(cnt) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false after `limit` SM cycles (2^28, about 0.13 s, unless a
// diagnostic launch asks for less).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, long long limit) {
  const long long t0 = clock64();
  while (!mbar_try_wait(b, parity)) {
    if (clock64() - t0 > limit) return false;
  }
  return true;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the shared-memory source of every committed store has been read
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// every committed store has completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void umma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), version 1 (bits 46-47).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)(16 >> 4) << 16;     // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;             // descriptor version
  d |= (uint64_t)2 << 61;             // SWIZZLE_128B
  return d;
}

// Instruction descriptor: D = F32, A/B format (BF16 = 1, TF32 = 2), K-major
// A and B, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t make_idesc(int ab_format, int M, int N) {
  return (1u << 4) | ((uint32_t)ab_format << 7) | ((uint32_t)ab_format << 10) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- activations (Instance.AssignActivation, TFInstance.py:108-140) ------
// The activation is a template parameter: a run-time switch over all five
// inlined into the 32-wide unrolled epilogue made the forward kernels
// instruction-fetch bound.
// The forward epilogue's activation h = act(z) and derivative act'(z) from
// one exponential, with the hardware exp2/log2 approximations (__expf,
// __logf: relative errors of a few 1e-7 on [1, 2] and below 1e-6 for exp's
// argument range here; the absolute error of h stays below 1e-9, far under
// the layer GEMM's). Four of the five activations spend most of the epilogue's
// instructions on these functions, and the epilogue has one warp per
// scheduler.
template <int ACT>
__device__ __forceinline__ void act_fwd(float z, float a, float& h, float& d) {
  if constexpr (ACT == TM_ACT_RELU) {
    h = fmaxf(z, 0.f);
    d = z > 0.f ? 1.f : 0.f;
  } else if constexpr (ACT == TM_ACT_SIGMOID_WITH_PARAM || ACT == TM_ACT_SOFTPLUS) {
    // log(1 + exp(t)) / a = (max(t, 0) + log1p(exp(-|t|))) / a, t = a z;
    // derivative sigmoid(t) = 1 / (1 + exp(-t))
    const float t = ACT == TM_ACT_SOFTPLUS ? z : a * z;
    const float e = __expf(-fabsf(t));
    const float ope = 1.f + e;
    const float l1p = ope == 1.f ? e : __logf(ope) * __fdividef(e, ope - 1.f);
    h = ACT == TM_ACT_SOFTPLUS ? fmaxf(t, 0.f) + l1p : __fdividef(fmaxf(t, 0.f) + l1p, a);
    d = __fdividef(t >= 0.f ? 1.f : e, ope);
  } else if constexpr (ACT == TM_ACT_TANH) {
    const float e = __expf(-2.f * fabsf(z));
    const float th = __fdividef(1.f - e, 1.f + e);
    h = copysignf(th, z);
    d = 1.f - th * th;
  } else {   // elu
    h = z > 0.f ? z : expm1f(z);
    d = z > 0.f ? 1.f : h + 1.f;
  }
}

// derivative expressed through the activation's output h = act(z)
template <int ACT>
__device__ __forceinline__ float actd_h(float h, float a) {
  if constexpr (ACT == TM_ACT_RELU) return h > 0.f ? 1.f : 0.f;
  if constexpr (ACT == TM_ACT_SIGMOID_WITH_PARAM) return -expm1f(-a * h);
  if constexpr (ACT == TM_ACT_SOFTPLUS) return -expm1f(-h);
  if constexpr (ACT == TM_ACT_TANH) return 1.f - h * h;
  return h > 0.f ? 1.f : h + 1.f;
}

template <int PREC>
struct Cfg {
  static constexpr int ELEM = PREC == TM_PREC_FP32 ? 4 : 2;
  static constexpr int BK = 128 / ELEM;               // one 128-byte swizzle row
  static constexpr int NSPLIT = PREC == TM_PREC_FP32 ? 2 : 1;
  static constexpr int BN = PREC == TM_PREC_FP32 ? 128 : 256;   // N tile
  static constexpr int NACC = NSPLIT;                 // accumulators per tile (main, correction)
  static constexpr int ACC_COLS = NACC * BN;          // TMEM columns per tile buffer: 256
  static constexpr int A_TILE = BM * 128;             // 16 KB
  static constexpr int B_TILE = BN * 128;             // 16 KB (tf32) or 32 KB (bf16)
  static constexpr int STAGE = NSPLIT * (A_TILE + B_TILE);   // 64 KB or 48 KB
  static constexpr int NSTAGE = PREC == TM_PREC_FP32 ? 3 : 4;
  // epilogue staging per epilogue warp (4 KB): FP32, a 32 x 32 box (hi parts,
  // then lo parts); BF16, a 32-row x 64-column box (or a 32 x 32 FP32 box for dE/dG)
  static constexpr int EPI_WB = 4096;
  static constexpr int EPI_BYTES = 8 * EPI_WB;
  static constexpr int SMEM = NSTAGE * STAGE + EPI_BYTES + 1024 + 256;   // + alignment, barriers
  static_assert((2 * NSTAGE + 4 + 8) * 8 + 8 <= 256, "barrier block");
  static constexpr uint32_t IDESC = make_idesc(PREC == TM_PREC_FP32 ? 2 : 1, BM, BN);
  // FP32: B hi and lo are adjacent 128-row tiles in a stage, i.e. one 256-row
  // operand, so A_hi [B_hi; B_lo] is a single N = 256 instruction writing the
  // main and the correction accumulator (adjacent in tensor memory)
  static constexpr uint32_t IDESC2 = make_idesc(2, BM, 2 * BN);
};

__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}

// Epilogue warps of one instantiation: eight (two per tensor-memory lane
// quarter, each with half of the tile's columns), except for the FP32 backward
// pass of a smooth activation, whose four warps bring the previous
// activation's hi and lo parts in with one bulk tensor load into an 8 KB box
// each (the same shared memory).
template <int PREC, int EPI, int ACT>
struct EpiShape {
  // the FP32 backward pass loads the previous activation into the staging
  // boxes (hi and lo side by side, 8 KB per warp), except with relu, whose
  // derivative comes from the forward pass's bits
  static constexpr bool BOXLOAD = PREC == TM_PREC_FP32 && EPI == EPI_BWD && ACT != TM_ACT_RELU;
  static constexpr int WARPS = (BOXLOAD && Cfg<PREC>::EPI_BYTES < 8 * 8192) ? 4 : 8;
  static constexpr int WB = Cfg<PREC>::EPI_BYTES / WARPS;   // staging bytes per warp
  static constexpr int THREADS = 32 * (WARPS + 2);
  // FP32: hi and lo boxes side by side (8 KB per warp), else one 4 KB box
  // that takes the hi parts, then the lo parts
  static constexpr bool PAIRBOX = PREC == TM_PREC_FP32 && WB >= 8192;
};

// Persistent, warp-specialised layer kernel. Each CTA walks tiles
// t = blockIdx.x, blockIdx.x + gridDim.x, ... in (net, m_tile, n_tile) order
// (n fastest, so the N-tiles of one M-tile run on neighbouring CTAs and share
// A through L2). The producer streams K-slices through the stage ring across
// tile boundaries; the MMA issuer alternates between two 256-column TMEM
// tile buffers, so the epilogue of tile t overlaps the MMAs of tile t + 1.
template <int PREC, int EPI, int ACT>
__global__ void __launch_bounds__(EpiShape<PREC, EPI, ACT>::THREADS, 1) k_gemm(const __grid_constant__ GemmArgs g) {
  using C = Cfg<PREC>;
  constexpr int BN = C::BN;
  constexpr bool KINK = PREC == TM_PREC_FP32 && ACT == TM_ACT_RELU && (EPI == EPI_FWD || EPI == EPI_FWD_LAST);
  // an earlier kernel of this context already failed: do nothing (every thread
  // reads the same word, written before this launch)
  if (*(volatile int*)&g.st->code != 0) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + C::NSTAGE * C::STAGE + C::EPI_BYTES);
  uint64_t* empty = full + C::NSTAGE;
  uint64_t* accf = empty + C::NSTAGE;   // [2] accumulator ready
  uint64_t* acce = accf + 2;            // [2] accumulator drained
  uint64_t* ebar = acce + 2;            // [8] previous-activation loads (FP32 backward),
                                        // one per epilogue warp
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(ebar + 8);
  constexpr int EW = EpiShape<PREC, EPI, ACT>::WARPS;
  constexpr bool BOXLOAD = EpiShape<PREC, EPI, ACT>::BOXLOAD;
  constexpr bool RMASK = ACT == TM_ACT_RELU && (EPI == EPI_FWD || EPI == EPI_BWD);
  // FP32 relu, last layer: the backward seed is act'(z) in {0, 1} (the output
  // weights are folded into the first backward launch's weights), one plane
  constexpr bool FOLD = PREC == TM_PREC_FP32 && ACT == TM_ACT_RELU && EPI == EPI_FWD_LAST;
  constexpr bool PAIRBOX = EpiShape<PREC, EPI, ACT>::PAIRBOX;
  static_assert(!BOXLOAD || PAIRBOX, "the FP32 backward pass loads hi and lo boxes together");
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = g.K / C::BK;
  const long long wlim = g.wait_limit > 0 ? g.wait_limit : (1LL << 28);
  const int per_net = g.mtiles * g.ntiles;
  const int total = 2 * per_net;

  if (threadIdx.x == 0) {
    for (int s = 0; s < C::NSTAGE; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], EW);   // one arrival per epilogue warp
    }
    for (int w = 0; w < 8; ++w) mbar_init(&ebar[w], 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(2 * C::ACC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == EW) {
    if (lane == 0) {
      int it = 0;
      for (int t = blockIdx.x; t < total && !*abort_flag; t += gridDim.x) {
        const int net = t / per_net, rem = t % per_net;
        const int m_tile = rem / g.ntiles, n_tile = rem % g.ntiles;
        const int elem = g.tile_elem[m_tile];
        const int a_row = net * g.a_net_rows + m_tile * BM;
        const int b_row = (net * g.nele + elem) * g.N + n_tile * BN;
        for (int kb = 0; kb < nk; ++kb, ++it) {
          const int s = it % C::NSTAGE;
          if (it >= C::NSTAGE && !mbar_wait(&empty[s], ((it / C::NSTAGE) - 1) & 1, wlim)) {
            tm_flag(g.st, TM_E_TIMEOUT, t, 100);
            *abort_flag = 1;
            break;
          }
          if (it == g.skip_it) continue;   // diagnostic: this stage never arrives
          uint8_t* st = smem + s * C::STAGE;
          mbar_expect_tx(&full[s], C::STAGE - (g.a_single ? C::A_TILE : 0));
          const int x = kb * C::BK;
          tma_load_2d(st, &g.a0, x, a_row, &full[s]);
          tma_load_2d(st + C::NSPLIT * C::A_TILE, &g.b0, x, b_row, &full[s]);
          if (C::NSPLIT == 2) {
            if (!g.a_single) tma_load_2d(st + C::A_TILE, &g.a1, x, a_row, &full[s]);
            tma_load_2d(st + 2 * C::A_TILE + C::B_TILE, &g.b1, x, b_row, &full[s]);
          }
        }
      }
    }
  } else if (warp == EW + 1) {
    if (lane == 0) {
      int it = 0, lt = 0;
      for (int t = blockIdx.x; t < total && !*abort_flag; t += gridDim.x, ++lt) {
        const int buf = lt & 1;
        if (lt >= 2 && !mbar_wait(&acce[buf], ((lt >> 1) - 1) & 1, wlim)) {
          tm_flag(g.st, TM_E_TIMEOUT, t, 103);
          *abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(buf * C::ACC_COLS);   // main; correction at + BN
        bool ok = true;
        for (int kb = 0; kb < nk; ++kb, ++it) {
          const int s = it % C::NSTAGE;
          if (!mbar_wait(&full[s], (it / C::NSTAGE) & 1, wlim)) {
            tm_flag(g.st, TM_E_TIMEOUT, t, 101);
            *abort_flag = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t base = smem_u32(smem + s * C::STAGE);
          const uint32_t a0 = base;
          const uint32_t a1 = base + C::A_TILE;
          const uint32_t b0 = base + C::NSPLIT * C::A_TILE;
          const uint32_t b1 = b0 + C::B_TILE;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            const uint64_t ad0 = sw128_desc(a0 + kk * 32), bd0 = sw128_desc(b0 + kk * 32);
            const uint32_t acc = (kb | kk) ? 1u : 0u;
            if (PREC == TM_PREC_FP32) {
              const uint64_t ad1 = sw128_desc(a1 + kk * 32);
              // A_hi B_hi -> main, A_hi B_lo -> correction (one instruction: A_hi is
              // read once), then A_lo B_hi -> correction
              umma_tf32(d, ad0, bd0, C::IDESC2, acc);
              if (!g.a_single) umma_tf32(d + BN, ad1, bd0, C::IDESC, 1u);
            } else {
              umma_f16(d, ad0, bd0, C::IDESC, acc);
            }
          }
          umma_commit(&empty[s]);
        }
        if (!ok) break;
        umma_commit(&accf[buf]);
      }
    }
  } else {
    // ---- epilogue: warps 0..7, thread = accumulator row ----
    // Two warps per tensor-memory lane quarter (warp w reads lanes 32 (w % 4)
    // ...), each taking half of the tile's columns: the epilogue's arithmetic
    // (activation, split, staging) outweighs the MMAs with one warp per
    // scheduler. Each warp stages 32 rows x 32 columns in shared memory in the
    // TMA 128-byte-swizzle layout (16-byte piece q of row r at piece q ^ (r &
    // 7): conflict-free for a row per lane) and writes them with bulk tensor
    // stores: FP32 hi then lo parts through one 4 KB box, BF16 64 columns per
    // box (two 32-column chunks). The backward pass reads the previous
    // activation of its rows with vector loads.
    const int quad = warp & 3, half = EW == 8 ? warp >> 2 : 0;
    constexpr int HALF = EW == 8 ? BN / 2 : BN;   // columns per warp
    float* ebox = reinterpret_cast<float*>(smem + C::NSTAGE * C::STAGE + warp * EpiShape<PREC, EPI, ACT>::WB);
    float* ebl = ebox + 1024;   // FP32 with 8 KB per warp: the lo box
    int eph = 0;                // uses of this warp's load barrier
    bool eok = true;
    int lt = 0;
    for (int t = blockIdx.x; t < total && eok; t += gridDim.x, ++lt) {
      const int buf = lt & 1;
      if (!mbar_wait(&accf[buf], (lt >> 1) & 1, wlim)) {
        tm_flag(g.st, TM_E_TIMEOUT, t, 102);
        *abort_flag = 1;
        break;
      }
      tc_fence_after();
      const int net = t / per_net, rem = t % per_net;
      const int m_tile = rem / g.ntiles, n_tile = rem % g.ntiles;
      const int elem = g.tile_elem[m_tile];
      const int row = m_tile * BM + quad * 32 + lane;          // row in this net
      const size_t orow = (size_t)net * g.Mpad + row;
      const int orow0 = net * g.Mpad + m_tile * BM + quad * 32;   // first row of this warp
      const int pblk = (net * g.nele + elem) * g.N;
      const int part = 2 * n_tile + half;                      // this warp's share of the row
      (void)part;
      const uint32_t tbase = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * C::ACC_COLS);
      float esum = 0.f;
      // relu refinement: kappa * ||input row|| (flags |z| below it times ||w_unit||)
      float kthr = 0.f, hss = 0.f;
      uint32_t kany = 0;   // flags of this thread's row in this warp's columns
      if constexpr (KINK) {
        if (g.kmask) {
          const float* pa = g.an2 + (size_t)net * g.an2_net_stride + (size_t)row * g.an2_parts;
          float ss = 0.f;
          for (int q = 0; q < g.an2_parts; ++q) ss += pa[q];
          kthr = g.kappa * sqrtf(ss);
        }
      }
      for (int c = half * HALF; c < (half + 1) * HALF && eok; c += 32) {
        const int col = n_tile * BN + c;
        // BF16 (not dE/dG): one 64-column box covers two 32-column chunks
        const bool box_start = PREC == TM_PREC_FP32 || EPI == EPI_OUT || (c & 32) == 0;
        const bool box_end = PREC == TM_PREC_FP32 || EPI == EPI_OUT || (c & 32) != 0;
        if (box_start) {
          // the staging box is free once the previous stores have read it
          if (lane == 0) bulk_wait_read();
          __syncwarp();
          if constexpr (BOXLOAD) {
            if (lane == 0) {
              mbar_expect_tx(&ebar[warp], 8192);
              tma_load_2d(ebox, &g.o0, col, orow0, &ebar[warp]);
              tma_load_2d(ebl, &g.o1, col, orow0, &ebar[warp]);
            }
          }
        }
        // the previous activation of these 32 columns (backward), then bias
        // and output weights (same for every row): loads issued before the
        // tensor-memory reads
        float h[32];
        uint32_t rbits = 0;   // relu backward: this row's bits of these 32 columns
        if constexpr (EPI == EPI_BWD && RMASK) rbits = g.rmask_in[orow * (g.N >> 5) + (col >> 5)];
        if constexpr (EPI == EPI_BWD && !BOXLOAD && !RMASK) {
          if constexpr (PREC == TM_PREC_FP32) {
            const float4* ph = reinterpret_cast<const float4*>(
                static_cast<const float*>(g.hprev0) + orow * g.ldo + col);
            const float4* pl = reinterpret_cast<const float4*>(
                static_cast<const float*>(g.hprev1) + orow * g.ldo + col);
            float4 a[8], b[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) { a[q] = ph[q]; b[q] = pl[q]; }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              h[4 * q] = a[q].x + b[q].x;
              h[4 * q + 1] = a[q].y + b[q].y;
              h[4 * q + 2] = a[q].z + b[q].z;
              h[4 * q + 3] = a[q].w + b[q].w;
            }
          } else {
            const uint4* ph = reinterpret_cast<const uint4*>(
                static_cast<const __nv_bfloat16*>(g.hprev0) + orow * g.ldo + col);
            uint4 u[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) u[q] = ph[q];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const uint32_t w[4] = {u[q].x, u[q].y, u[q].z, u[q].w};
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[e]));
                h[8 * q + 2 * e] = f.x;
                h[8 * q + 2 * e + 1] = f.y;
              }
            }
          }
        }
        // bias, output weight and (relu refinement) unit norm of these 32
        // columns, the same for every row: lane q holds column q's values and
        // the loop takes them by shuffle (one coalesced load each, issued
        // before the tensor-memory reads; 32-float register copies spill)
        float b_l = 0.f, w_l = 0.f, wn_l = 0.f;
        if (EPI == EPI_FWD || EPI == EPI_FWD_LAST) b_l = __ldg(g.bias + pblk + col + lane);
        if (EPI == EPI_FWD_LAST) w_l = __ldg(g.wout + pblk + col + lane);
        if constexpr (KINK) {
          if (g.kmask) wn_l = __ldg(g.wnorm + pblk + col + lane);
        }
        uint32_t r[32];
        tmem_ld32(tbase + (uint32_t)c, r);
        if (C::NACC == 2) {
          uint32_t r2[32];
          tmem_ld32(tbase + (uint32_t)(BN + c), r2);
#pragma unroll
          for (int q = 0; q < 32; ++q)
            r[q] = __float_as_uint(__uint_as_float(r[q]) + __uint_as_float(r2[q]));
        }
        float v[32];
        if (EPI == EPI_FWD || EPI == EPI_FWD_LAST) {
          uint32_t km = 0, rm = 0;
#pragma unroll
          for (int q = 0; q < 32; ++q) {
            const float z = __uint_as_float(r[q]) + __shfl_sync(TM_FULL, b_l, q);
            if constexpr (KINK) {
              if (fabsf(z) < kthr * __shfl_sync(TM_FULL, wn_l, q)) km |= 1u << q;
            }
            float hz, dz;
            act_fwd<ACT>(z, g.alpha, hz, dz);
            if (EPI == EPI_FWD) {
              v[q] = hz;
              if constexpr (RMASK) rm |= (hz > 0.f ? 1u : 0u) << q;
              if constexpr (KINK) hss = fmaf(v[q], v[q], hss);
            } else {
              const float wq = __shfl_sync(TM_FULL, w_l, q);
              esum += hz * wq;
              v[q] = FOLD ? dz : wq * dz;
            }
          }
          if constexpr (RMASK && EPI == EPI_FWD) {
            if (g.rmask_out) g.rmask_out[orow * (g.N >> 5) + (col >> 5)] = rm;
          }
          if constexpr (KINK) {
            if (g.kmask) g.kmask[((size_t)net * g.Mpad + row) * (g.N >> 5) + (col >> 5)] = km;
            kany |= km;
          }
        } else if (EPI == EPI_BWD) {
          if constexpr (BOXLOAD) {
            if (!mbar_wait(&ebar[warp], eph & 1, wlim)) {
              tm_flag(g.st, TM_E_TIMEOUT, t, 104);
              *abort_flag = 1;
              eok = false;
            }
            ++eph;
            const float4* sh = reinterpret_cast<const float4*>(ebox) + lane * 8;
            const float4* sl = reinterpret_cast<const float4*>(ebl) + lane * 8;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const float4 a = sh[q ^ (lane & 7)], b = sl[q ^ (lane & 7)];
              h[4 * q] = a.x + b.x;
              h[4 * q + 1] = a.y + b.y;
              h[4 * q + 2] = a.z + b.z;
              h[4 * q + 3] = a.w + b.w;
            }
            __syncwarp();   // every lane has read the boxes before they take the outputs
          }
          if constexpr (RMASK) {
#pragma unroll
            for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]) * (((rbits >> q) & 1u) ? 1.f : 0.f);
          } else {
#pragma unroll
            for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]) * actd_h<ACT>(h[q], g.alpha);
          }
        } else {
#pragma unroll
          for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
        }
        float4* dh = reinterpret_cast<float4*>(ebox) + lane * 8;
        if constexpr (PREC == TM_PREC_FP32) {
          if constexpr (EPI == EPI_OUT) {   // one FP32 output
#pragma unroll
            for (int q = 0; q < 8; ++q)
              dh[q ^ (lane & 7)] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
          } else if constexpr (PAIRBOX) {   // hi and lo boxes side by side
            float4* dl = reinterpret_cast<float4*>(ebl) + lane * 8;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              float4 hh, ll;
              tm_tf32_split(v[4 * q], hh.x, ll.x);
              tm_tf32_split(v[4 * q + 1], hh.y, ll.y);
              tm_tf32_split(v[4 * q + 2], hh.z, ll.z);
              tm_tf32_split(v[4 * q + 3], hh.w, ll.w);
              dh[q ^ (lane & 7)] = hh;
              dl[q ^ (lane & 7)] = ll;
            }
          } else {                          // hi parts now, lo parts after them
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              float4 hh;
              hh.x = tm_tf32_rn(v[4 * q]);
              hh.y = tm_tf32_rn(v[4 * q + 1]);
              hh.z = tm_tf32_rn(v[4 * q + 2]);
              hh.w = tm_tf32_rn(v[4 * q + 3]);
              dh[q ^ (lane & 7)] = hh;
            }
          }
          fence_async_smem();
          __syncwarp();
          if (lane == 0) {
            tma_store_2d(&g.o0, col, orow0, ebox);
            if (PAIRBOX && EPI != EPI_OUT) tma_store_2d(&g.o1, col, orow0, ebl);
            bulk_commit();
          }
          if constexpr (EPI != EPI_OUT && !PAIRBOX && !FOLD) {
            if (lane == 0) bulk_wait_read();
            __syncwarp();
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              float4 ll;
              ll.x = tm_tf32_rn(v[4 * q] - tm_tf32_rn(v[4 * q]));
              ll.y = tm_tf32_rn(v[4 * q + 1] - tm_tf32_rn(v[4 * q + 1]));
              ll.z = tm_tf32_rn(v[4 * q + 2] - tm_tf32_rn(v[4 * q + 2]));
              ll.w = tm_tf32_rn(v[4 * q + 3] - tm_tf32_rn(v[4 * q + 3]));
              dh[q ^ (lane & 7)] = ll;
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0) {
              tma_store_2d(&g.o1, col, orow0, ebox);
              bulk_commit();
            }
          }
        } else if (EPI == EPI_OUT) {
          // FP32 dE/dG through a 32 x 32 FP32 box
#pragma unroll
          for (int q = 0; q < 8; ++q)
            dh[q ^ (lane & 7)] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
          fence_async_smem();
          __syncwarp();
          if (lane == 0) {
            tma_store_2d(&g.o0, col, orow0, ebox);   // the FP32 map of dE/dG
            bulk_commit();
          }
        } else {
          uint4* db = reinterpret_cast<uint4*>(ebox) + lane * 8;
          const int p0 = (c & 32) ? 4 : 0;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            __nv_bfloat162 b[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) b[e] = __floats2bfloat162_rn(v[8 * q + 2 * e], v[8 * q + 2 * e + 1]);
            db[(p0 + q) ^ (lane & 7)] =
                make_uint4(*reinterpret_cast<uint32_t*>(&b[0]), *reinterpret_cast<uint32_t*>(&b[1]),
                           *reinterpret_cast<uint32_t*>(&b[2]), *reinterpret_cast<uint32_t*>(&b[3]));
          }
          if (box_end) {
            fence_async_smem();
            __syncwarp();
            if (lane == 0) {
              tma_store_2d(&g.o0, col - 32, orow0, ebox);
              bulk_commit();
            }
          }
        }
      }
      if (EPI == EPI_FWD_LAST) g.epart[orow * (2 * g.ntiles) + part] = esum;
      if constexpr (KINK) {
        // (row, column part) entries with flagged units, for the refinement:
        // one atomic per warp
        const uint32_t bal = __ballot_sync(TM_FULL, kany != 0u);
        if (bal && g.kmask) {
          uint32_t base = 0;
          if (lane == 0) base = atomicAdd(g.knrows, (uint32_t)__popc(bal));
          base = __shfl_sync(TM_FULL, base, 0);
          if (kany) g.krows[base + __popc(bal & ((1u << lane) - 1u))] = (uint32_t)(orow * (2 * g.ntiles) + part);
        }
      }
      if constexpr (KINK && EPI == EPI_FWD) {
        if (g.hn2_out) g.hn2_out[orow * (2 * g.ntiles) + part] = hss;
      }
      // this warp has read its lanes and columns of the accumulator: hand them back
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[buf]);
    }
    if (lane == 0) bulk_wait_all();
    __syncwarp();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * C::ACC_COLS)
                 : "memory");
  }
}

template <int PREC, int EPI, int ACT>
int launch_gemm(tm_ctx* ctx, const GemmArgs& g0, int mtiles) {
  using C = Cfg<PREC>;
  if (g0.N % C::BN) return tm_fail(ctx, TM_E_ARG, "gemm width not a multiple of the N tile");
  const int ntiles = g0.N / C::BN;
  static bool attr_set = false;   // the shared-memory size is fixed per instantiation
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_gemm<PREC, EPI, ACT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    if (e != cudaSuccess) return tm_cuda_check(ctx, e, "gemm attr");
    attr_set = true;
  }
  GemmArgs g = g0;
  g.mtiles = mtiles;
  g.ntiles = ntiles;
  const int total = 2 * mtiles * ntiles;
  const int grid = total < ctx->num_sms ? total : ctx->num_sms;
  k_gemm<PREC, EPI, ACT><<<grid, EpiShape<PREC, EPI, ACT>::THREADS, C::SMEM, ctx->stream>>>(g);
  ctx->launches++;
  return tm_cuda_check(ctx, cudaGetLastError(), "gemm");
}

template <int PREC, int ACT>
int run_gemm(tm_ctx* ctx, int epi, const GemmArgs& g, int mtiles) {
  switch (epi) {
    case EPI_FWD: return launch_gemm<PREC, EPI_FWD, ACT>(ctx, g, mtiles);
    case EPI_FWD_LAST: return launch_gemm<PREC, EPI_FWD_LAST, ACT>(ctx, g, mtiles);
    case EPI_BWD: return launch_gemm<PREC, EPI_BWD, ACT>(ctx, g, mtiles);
    default: return launch_gemm<PREC, EPI_OUT, TM_ACT_RELU>(ctx, g, mtiles);
  }
}

template <int PREC>
int run_gemm_act(tm_ctx* ctx, int epi, const GemmArgs& g, int mtiles) {
  switch (epi == EPI_OUT ? TM_ACT_RELU : g.act) {
    case TM_ACT_RELU: return run_gemm<PREC, TM_ACT_RELU>(ctx, epi, g, mtiles);
    case TM_ACT_SIGMOID_WITH_PARAM: return run_gemm<PREC, TM_ACT_SIGMOID_WITH_PARAM>(ctx, epi, g, mtiles);
    case TM_ACT_SOFTPLUS: return run_gemm<PREC, TM_ACT_SOFTPLUS>(ctx, epi, g, mtiles);
    case TM_ACT_TANH: return run_gemm<PREC, TM_ACT_TANH>(ctx, epi, g, mtiles);
    case TM_ACT_ELU: return run_gemm<PREC, TM_ACT_ELU>(ctx, epi, g, mtiles);
    default: return tm_fail(ctx, TM_E_ARG, "activation");
  }
}

int dispatch(tm_ctx* ctx, int prec, int epi, const GemmArgs& g, int mtiles) {
  return prec == TM_PREC_FP32 ? run_gemm_act<TM_PREC_FP32>(ctx, epi, g, mtiles)
                              : run_gemm_act<TM_PREC_BF16>(ctx, epi, g, mtiles);
}

// ---- relu refinement --------------------------------------------------------
// The tensor core's FP32 accumulation truncates at every instruction, which
// puts the pre-activation z of a unit up to about (K/8) 2^-23 sum|a||w| away
// from its exact value. A relu unit whose z lies that close to zero can take
// the other side of the kink, and its derivative (0 or 1) then differs from
// the exact network's: the force jumps. The forward epilogue flags every unit
// with |z| < kappa ||a|| ||w|| (Cauchy-Schwarz: ||a|| ||w|| >= sum|a||w|), and
// this kernel recomputes the flagged ones from the layer's stored input
// (hi + lo, an exact sum) and the weights and bias as given (FP64, held as
// double-single pairs), with a double-single dot product (TwoProduct and
// TwoSum per term, Ogita, Rump and Oishi 2005), then rewrites the unit's
// output: h = relu(z) for a hidden layer, w_out * step(z) (the backward pass's
// seed) for the last one. The energy of the last layer keeps the tensor-core z
// of a flagged unit (a change below kappa ||a|| ||w|| |w_out|).
struct KinkArgs {
  const float* a_hi;
  const float* a_lo;
  int a_net_rows;         // 0: both nets read the same input rows (the descriptors)
  int K;
  const float2* w2;       // [2][nele][N][K] (hi, lo)
  const float2* b2;       // [2][nele][N]
  const float* wout;      // [2][nele][N]
  const int32_t* tile_elem;
  const uint32_t* kmask;  // [2][Mpad][N/32]
  uint32_t* rmask;        // hidden layers: the relu bits the backward pass reads (or null)
  int fold;               // last layer: write act'(z) (the output weights are folded), hi only
  const uint32_t* rows;   // entries orow * parts + part (appended by the layer kernel)
  const uint32_t* nrows;
  int parts, part_cols;   // column parts per row and their width
  float* o_hi;
  float* o_lo;            // [2*Mpad][N]
  int N, Mpad, nele;
  unsigned long long* count;
};

// Persistent warps over the entries (row, column part) that the layer kernel
// flagged. An entry reads its row's input once into registers (KPL values per
// lane, all loads in flight together); each flagged unit of the part then
// streams its weight vector with independent loads.
template <bool LAST, int KPL>
__global__ void __launch_bounds__(256) k_kink_refine(const KinkArgs a) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (int)((gridDim.x * (size_t)blockDim.x) >> 5);
  const int n = (int)*a.nrows;
  int nref = 0;
  for (int e = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5); e < n; e += nwarps) {
    const uint32_t ent = a.rows[e];
    const int orow = (int)(ent / (uint32_t)a.parts), part = (int)(ent % (uint32_t)a.parts);
    const int net = orow / a.Mpad, r = orow - net * a.Mpad;
    const int c0 = part * a.part_cols;
    const uint32_t* mk = a.kmask + (size_t)orow * (a.N >> 5) + (c0 >> 5);
    const uint32_t mine = lane < (a.part_cols >> 5) ? mk[lane] : 0u;   // one flag word per lane
    const int elem = a.tile_elem[r / BM];
    const size_t blk = (size_t)net * a.nele + elem;
    const size_t arow = (size_t)net * a.a_net_rows + r;
    const float* ah = a.a_hi + arow * a.K + lane;
    const float* al = a.a_lo + arow * a.K + lane;
    constexpr int KR = KPL > 0 ? KPL : 1;
    float xh[KR], xl[KR];
#pragma unroll
    for (int q = 0; q < KPL; ++q) {
      xh[q] = ah[q * 32];
      xl[q] = al[q * 32];
    }
    uint32_t any = __ballot_sync(TM_FULL, mine != 0u);
    while (any) {
      const int src = __ffs(any) - 1;
      any &= any - 1;
      uint32_t bits = __shfl_sync(TM_FULL, mine, src);
      while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1;
        const int col = c0 + src * 32 + b;
        const float2* wr = a.w2 + (blk * a.N + col) * a.K + lane;
        float sh = 0.f, sl = 0.f;
        if constexpr (KPL > 0) {
          float2 wv[KPL];
#pragma unroll
          for (int q = 0; q < KPL; ++q) wv[q] = __ldg(wr + q * 32);
#pragma unroll
          for (int q = 0; q < KPL; ++q) {
            float p, e2, t;
            tm_two_prod(xh[q], wv[q].x, p, e2);
            tm_two_sum(sh, p, sh, t);
            sl += (t + e2) + fmaf(xh[q], wv[q].y, xl[q] * wv[q].x);
          }
        } else {   // any K that is a multiple of 32: the input streamed as well
#pragma unroll 8
          for (int q = 0; q < a.K / 32; ++q) {
            const float2 wq = __ldg(wr + q * 32);
            const float x = ah[q * 32], xq = al[q * 32];
            float p, e2, t;
            tm_two_prod(x, wq.x, p, e2);
            tm_two_sum(sh, p, sh, t);
            sl += (t + e2) + fmaf(x, wq.y, xq * wq.x);
          }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
          const float oh = __shfl_xor_sync(TM_FULL, sh, o), ol = __shfl_xor_sync(TM_FULL, sl, o);
          float t;
          tm_two_sum(sh, oh, sh, t);
          sl += t + ol;
        }
        if (lane == 0) {
          const float2 bb = a.b2[blk * a.N + col];
          float t;
          tm_two_sum(sh, bb.x, sh, t);
          sl += t + bb.y;
          const float z = sh + sl;
          const float v = LAST ? (z > 0.f ? (a.fold ? 1.f : a.wout[blk * a.N + col]) : 0.f)
                               : (z > 0.f ? z : 0.f);
          float hi, lo;
          tm_tf32_split(v, hi, lo);
          const size_t o = ((size_t)net * a.Mpad + r) * a.N + col;
          a.o_hi[o] = hi;
          if (!(LAST && a.fold)) a.o_lo[o] = lo;
          if (!LAST && a.rmask) {
            unsigned int* wd = a.rmask + (o >> 5);
            const unsigned int bit = 1u << (col & 31);
            if (z > 0.f) atomicOr(wd, bit);
            else atomicAnd(wd, ~bit);
          }
        }
        ++nref;
      }
    }
  }
  if (lane == 0 && nref && a.count) atomicAdd(a.count, (unsigned long long)nref);
}

template <bool LAST>
int launch_kink_refine(tm_ctx* ctx, const KinkArgs& ka) {
  const int blocks = 4 * ctx->num_sms;   // persistent: a few thousand entries per layer
  switch (ka.K / 32) {
    case 8: k_kink_refine<LAST, 8><<<blocks, 256, 0, ctx->stream>>>(ka); break;
    case 16: k_kink_refine<LAST, 16><<<blocks, 256, 0, ctx->stream>>>(ka); break;
    case 24: k_kink_refine<LAST, 24><<<blocks, 256, 0, ctx->stream>>>(ka); break;
    case 32: k_kink_refine<LAST, 32><<<blocks, 256, 0, ctx->stream>>>(ka); break;
    default: k_kink_refine<LAST, 0><<<blocks, 256, 0, ctx->stream>>>(ka); break;
  }
  ctx->launches++;
  return tm_cuda_check(ctx, cudaGetLastError(), "relu refinement");
}

}  // namespace

// kappa of the flag test for a reduction of length K: (K/8) 2^-23 for the
// truncations of the main accumulator (one per 8-deep tf32 instruction) plus
// 8 2^-23 for the split operands' residuals and the correction accumulator
float tm_kink_kappa(int K) { return (float)((K / 8 + 8) * 0x1p-23); }

int tm_gemm_bn(int prec) {
  return prec == TM_PREC_FP32 ? Cfg<TM_PREC_FP32>::BN : Cfg<TM_PREC_BF16>::BN;
}

// partial row sums a layer launch writes per row (energy, squared norms): one
// per N tile and column half
int tm_gemm_row_parts(int prec, int H) { return 2 * (H / tm_gemm_bn(prec)); }

int tm_make_tmap(tm_ctx* ctx, CUtensorMap* map, void* base, int elem_bytes, uint64_t rows,
                 uint64_t cols, uint32_t box_rows) {
  if (!ctx->encode) return tm_fail(ctx, TM_E_CUDA, "cuTensorMapEncodeTiled unavailable");
  const CUtensorMapDataType dt =
      elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * (cuuint64_t)elem_bytes};
  cuuint32_t box[2] = {(cuuint32_t)(128 / elem_bytes), box_rows};
  cuuint32_t es[2] = {1, 1};
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (strides[0] & 15))
    return tm_fail(ctx, TM_E_ARG, "tensor map alignment");
  CUresult r = ctx->encode(map, dt, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return tm_fail(ctx, TM_E_CUDA, "cuTensorMapEncodeTiled failed");
  return TM_OK;
}

// Six launches per energy+force (both networks per launch):
//   fwd 0..L-1 (last one: energy dot product + g_L = w_out * act'(z_L)),
//   bwd L-1..1 (g_{l-1} = (g_l W_l^T) * act'(z_{l-1}), in place over h_{l-1}),
//   bwd 0 (dE/dG = g_1 W_1^T, FP32).
// ev (optional): 2 events per layer GEMM launch, recorded around it (forward
// layers first, then backward), for tm_system_profile_layers.
static int mlp_layers(tm_system* s, bool forward, bool backward, cudaEvent_t* ev = nullptr);

int tm_launch_mlp(tm_system* s, bool backward) { return mlp_layers(s, true, backward); }
int tm_launch_mlp_backward_only(tm_system* s) { return mlp_layers(s, false, true); }

int tm_profile_layers(tm_system* s, float* ms) {
  tm_ctx* ctx = s->ctx;
  const int L = s->model->nlayer;
  std::vector<cudaEvent_t> ev(4 * L);
  for (auto& e : ev) cudaEventCreate(&e);
  int rc = mlp_layers(s, true, true, ev.data());
  if (!rc) rc = tm_cuda_check(ctx, cudaEventSynchronize(ev[4 * L - 1]), "profile layers");
  if (!rc)
    for (int q = 0; q < 2 * L; ++q) cudaEventElapsedTime(&ms[q], ev[2 * q], ev[2 * q + 1]);
  for (auto& e : ev) cudaEventDestroy(e);
  if (!rc) rc = tm_sync_status(ctx, "profile layers");
  return rc;
}

static int mlp_layers(tm_system* s, bool forward, bool backward, cudaEvent_t* ev) {
  tm_model* m = s->model;
  tm_ctx* ctx = s->ctx;
  const int L = m->nlayer;
  const int H = m->H, Dp = m->k.Dp;
  const int mt = s->ntiles;
  const int prec = m->desc.precision;
  int rc;
  // activation buffers: level 0 = G (shared), levels 1..L-1 = H_l, level L = g_L
  const CUtensorMap* lv0[2] = {&s->tm_G[0], &s->tm_G[1]};
  const CUtensorMap* lvH[TM_MAX_HIDDEN][2] = {{&s->tm_H1[0], &s->tm_H1[1]},
                                              {&s->tm_H2[0], &s->tm_H2[1]}};
  void* bufH[TM_MAX_HIDDEN][2] = {{s->H1[0], s->H1[1]}, {s->H2[0], s->H2[1]}};
  // 32-row store boxes of the same buffers (FP32 mode)
  const CUtensorMap* stH[TM_MAX_HIDDEN][2] = {{&s->ts_H1[0], &s->ts_H1[1]},
                                              {&s->ts_H2[0], &s->ts_H2[1]}};
  GemmArgs g;
  memset(&g, 0, sizeof(g));
  g.nele = m->k.nele;
  g.tile_elem = s->tile_elem;
  g.Mpad = s->Mpad;
  g.act = m->k.act;
  g.alpha = m->k.alpha_sig;
  g.st = ctx->d_status;
  g.skip_it = -1;
  const bool kink = m->kink && s->kink_mask;
  // FP32 relu: the last forward layer writes act'(z) for the folded backward
  // weights (a choice the kernel makes at compile time), so they must exist
  if (prec == TM_PREC_FP32 && m->k.act == TM_ACT_RELU && !m->w_bwd_fold[0])
    return tm_fail(ctx, TM_E_STATE, "relu model without its folded backward weights");
  const int nparts = tm_gemm_row_parts(prec, H);
  if (forward && kink && s->kink_count) {
    cudaMemsetAsync(s->kink_count, 0, sizeof(unsigned long long), ctx->stream);
    cudaMemsetAsync(s->kink_nrows, 0, sizeof(uint32_t) * TM_KINK_LAYERS, ctx->stream);
  }
  for (int l = 0; forward && l < L; ++l) {
    const bool last = (l == L - 1);
    const CUtensorMap* const* A = l == 0 ? lv0 : lvH[l - 1];
    g.a0 = *A[0];
    g.a1 = *A[1];
    g.b0 = m->tm_wf[l][0];
    g.b1 = m->tm_wf[l][1];
    g.K = l == 0 ? Dp : H;
    g.N = H;
    g.a_net_rows = l == 0 ? 0 : s->Mpad;
    g.bias = m->bias[l];
    g.wout = m->wout;
    g.epart = s->epart;
    g.ldo = H;
    g.out0 = last ? s->G3[0] : bufH[l][0];
    g.out1 = last ? s->G3[1] : bufH[l][1];
    g.o0 = last ? s->ts_G3[0] : *stH[l][0];
    g.o1 = last ? s->ts_G3[1] : *stH[l][1];
    g.rmask_out = (m->k.act == TM_ACT_RELU && !last && s->relu_mask)
                      ? s->relu_mask + (size_t)l * 2 * s->Mpad * (H / 32) : nullptr;
    if (kink) {
      g.kmask = s->kink_mask;
      g.wnorm = m->kwn[l];
      g.kappa = tm_kink_kappa(g.K);
      g.an2 = l == 0 ? s->kink_g2 : s->kink_h2[(l - 1) & 1];
      g.an2_parts = l == 0 ? 1 : nparts;
      g.an2_net_stride = l == 0 ? 0 : s->Mpad * nparts;
      g.hn2_out = last ? nullptr : s->kink_h2[l & 1];
      g.krows = s->kink_rows;
      g.knrows = s->kink_nrows + l;
    }
    if (ev) cudaEventRecord(ev[2 * l], ctx->stream);
    if ((rc = dispatch(ctx, prec, last ? EPI_FWD_LAST : EPI_FWD, g, mt))) return rc;
    if (ev) cudaEventRecord(ev[2 * l + 1], ctx->stream);
    if (kink) {
      KinkArgs ka;
      ka.a_hi = static_cast<const float*>(l == 0 ? s->G[0] : bufH[l - 1][0]);
      ka.a_lo = static_cast<const float*>(l == 0 ? s->G[1] : bufH[l - 1][1]);
      ka.a_net_rows = l == 0 ? 0 : s->Mpad;
      ka.K = g.K;
      ka.w2 = m->kw2[l];
      ka.b2 = m->kb2[l];
      ka.wout = m->wout;
      ka.tile_elem = s->tile_elem;
      ka.kmask = s->kink_mask;
      ka.o_hi = static_cast<float*>(last ? s->G3[0] : bufH[l][0]);
      ka.o_lo = static_cast<float*>(last ? s->G3[1] : bufH[l][1]);
      ka.N = H;
      ka.Mpad = s->Mpad;
      ka.nele = m->k.nele;
      ka.count = s->kink_count;
      ka.rmask = g.rmask_out;
      ka.fold = last && m->w_bwd_fold[0] ? 1 : 0;
      ka.rows = s->kink_rows;
      ka.nrows = s->kink_nrows + l;
      ka.parts = nparts;
      ka.part_cols = H / nparts;
      if ((rc = last ? launch_kink_refine<true>(ctx, ka) : launch_kink_refine<false>(ctx, ka))) return rc;
    }
  }
  g.kmask = nullptr;
  g.hn2_out = nullptr;
  g.rmask_out = nullptr;
  if (!backward) return TM_OK;
  for (int l = L - 1; l >= 0; --l) {
    // A = g_{l+1} (level l+1 buffer), B = W_l as [Kin x Nout] rows
    const CUtensorMap* gA[2];
    if (l == L - 1) { gA[0] = &s->tm_G3[0]; gA[1] = &s->tm_G3[1]; }
    else { gA[0] = lvH[l][0]; gA[1] = lvH[l][1]; }
    g.a0 = *gA[0];
    g.a1 = *gA[1];
    g.b0 = m->tm_wb[l][0];
    g.b1 = m->tm_wb[l][1];
    g.a_single = 0;
    if (l == L - 1 && m->w_bwd_fold[0]) {   // FP32 relu: seed act'(z), w_out folded into W
      g.b0 = m->tm_wbf[0];
      g.b1 = m->tm_wbf[1];
      g.a_single = 1;
    }
    g.K = H;
    g.a_net_rows = s->Mpad;
    if (l > 0) {
      g.N = H;
      g.ldo = H;
      g.hprev0 = bufH[l - 1][0];
      g.hprev1 = bufH[l - 1][1];
      g.rmask_in = (m->k.act == TM_ACT_RELU && s->relu_mask)
                       ? s->relu_mask + (size_t)(l - 1) * 2 * s->Mpad * (H / 32) : nullptr;
      g.out0 = bufH[l - 1][0];
      g.out1 = bufH[l - 1][1];
      g.o0 = *stH[l - 1][0];
      g.o1 = *stH[l - 1][1];
      if (ev) cudaEventRecord(ev[2 * (2 * L - 1 - l)], ctx->stream);
      if ((rc = dispatch(ctx, prec, EPI_BWD, g, mt))) return rc;
      if (ev) cudaEventRecord(ev[2 * (2 * L - 1 - l) + 1], ctx->stream);
    } else {
      g.N = Dp;
      g.ldo = Dp;
      g.out0 = s->dEdG;
      g.out1 = nullptr;
      g.o0 = s->ts_dEdG;
      if (ev) cudaEventRecord(ev[2 * (2 * L - 1)], ctx->stream);
      if ((rc = dispatch(ctx, prec, EPI_OUT, g, mt))) return rc;
      if (ev) cudaEventRecord(ev[2 * (2 * L - 1) + 1], ctx->stream);
    }
  }
  return TM_OK;
}

// Stand-alone check of the tensor-core path: C[M,N] = A[M,K] B[N,K]^T with a
// single element and net 0 (host fp32 in/out). Used by the GPU tests.
int tm_gemm_selftest(tm_ctx* ctx, int prec, int M, int N, int K, const float* A, const float* B,
                     float* Cout, long long wait_limit, int skip_it) {
  const int BN = tm_gemm_bn(prec);
  if (M % BM || N % BN || K % 64) return tm_fail(ctx, TM_E_ARG, "selftest shape");
  const int eb = prec == TM_PREC_FP32 ? 4 : 2;
  const size_t nA = (size_t)M * K, nB = (size_t)N * K, nC = (size_t)M * N;
  std::vector<uint8_t> ha0(nA * eb), ha1(nA * eb), hb0(nB * eb), hb1(nB * eb);
  auto split = [&](const float* src, size_t n, uint8_t* d0, uint8_t* d1) {
    for (size_t q = 0; q < n; ++q) {
      if (prec == TM_PREC_FP32) {
        float h, lo;
        tm_tf32_split(src[q], h, lo);
        memcpy(d0 + 4 * q, &h, 4);
        memcpy(d1 + 4 * q, &lo, 4);
      } else {
        __nv_bfloat16 b = __float2bfloat16_rn(src[q]);
        memcpy(d0 + 2 * q, &b, 2);
      }
    }
  };
  split(A, nA, ha0.data(), ha1.data());
  split(B, nB, hb0.data(), hb1.data());
  // stack two copies of B rows so that net 1 (unused output) stays in bounds
  void *da0, *da1, *db0, *db1, *dc, *dc1, *dbias, *dw;
  int32_t* dte;
  tm_dev_status* st = ctx->d_status;
  int rc = 0;
  if ((rc = tm_alloc(ctx, &da0, nA * eb * 2)) || (rc = tm_alloc(ctx, &da1, nA * eb * 2)) ||
      (rc = tm_alloc(ctx, &db0, nB * eb * 2)) || (rc = tm_alloc(ctx, &db1, nB * eb * 2)) ||
      (rc = tm_alloc(ctx, &dc, nC * 4 * 2)) || (rc = tm_alloc(ctx, &dc1, nC * 4 * 2)) ||
      (rc = tm_alloc(ctx, &dbias, (size_t)N * 4 * 2)) || (rc = tm_alloc(ctx, &dw, (size_t)N * 4 * 2)) ||
      (rc = tm_alloc(ctx, (void**)&dte, sizeof(int32_t) * (M / BM))))
    return rc;
  cudaStream_t sm = ctx->stream;
  for (int c = 0; c < 2; ++c) {
    cudaMemcpyAsync((uint8_t*)da0 + c * nA * eb, ha0.data(), nA * eb, cudaMemcpyHostToDevice, sm);
    cudaMemcpyAsync((uint8_t*)da1 + c * nA * eb, ha1.data(), nA * eb, cudaMemcpyHostToDevice, sm);
    cudaMemcpyAsync((uint8_t*)db0 + c * nB * eb, hb0.data(), nB * eb, cudaMemcpyHostToDevice, sm);
    cudaMemcpyAsync((uint8_t*)db1 + c * nB * eb, hb1.data(), nB * eb, cudaMemcpyHostToDevice, sm);
  }
  cudaMemsetAsync(dte, 0, sizeof(int32_t) * (M / BM), sm);
  GemmArgs g;
  memset(&g, 0, sizeof(g));
  if ((rc = tm_make_tmap(ctx, &g.a0, da0, eb, 2 * (uint64_t)M, K, BM)) ||
      (rc = tm_make_tmap(ctx, &g.a1, prec == TM_PREC_FP32 ? da1 : da0, eb, 2 * (uint64_t)M, K, BM)) ||
      (rc = tm_make_tmap(ctx, &g.b0, db0, eb, 2 * (uint64_t)N, K, BN)) ||
      (rc = tm_make_tmap(ctx, &g.b1, prec == TM_PREC_FP32 ? db1 : db0, eb, 2 * (uint64_t)N, K, BN)) ||
      (rc = tm_make_tmap(ctx, &g.o0, dc, 4, 2 * (uint64_t)M, N, 32)))
    return rc;
  g.K = K; g.N = N; g.a_net_rows = M; g.nele = 1; g.tile_elem = dte; g.Mpad = M;
  g.out0 = dc; g.out1 = dc1; g.ldo = N; g.st = st;
  g.wait_limit = wait_limit;
  g.skip_it = skip_it;
  rc = dispatch(ctx, prec, EPI_OUT, g, M / BM);
  if (!rc) rc = tm_cuda_check(ctx, cudaMemcpyAsync(Cout, dc, nC * 4, cudaMemcpyDeviceToHost, sm), "selftest d2h");
  if (!rc) rc = tm_sync_status(ctx, "gemm selftest");
  tm_free(ctx, da0, nA * eb * 2); tm_free(ctx, da1, nA * eb * 2);
  tm_free(ctx, db0, nB * eb * 2); tm_free(ctx, db1, nB * eb * 2);
  tm_free(ctx, dc, nC * 8); tm_free(ctx, dc1, nC * 8);
  tm_free(ctx, dbias, (size_t)N * 8); tm_free(ctx, dw, (size_t)N * 8);
  tm_free(ctx, dte, sizeof(int32_t) * (M / BM));
  return rc;
}
