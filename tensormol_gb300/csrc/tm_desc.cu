// ANI-1 symmetry functions (forward) and their Jacobian-transpose (adjoint).
//
// Forward follows TFSymRSet_Linear_WithEle_Release (TFDescriptors/RawSymFunc.py:
// 1757-1810) and TFSymASet_Linear_WithEle (RawSymFunc.py:868-963), assembled as
// in TFSymSet_Scattered_Linear_WithEle_Release (RawSymFunc.py:2267-2309):
//   row = [ radial: element-major, AN1_num_r_Rs shifts
//         | angular: element-pair-major, theta-major (8), then Rs (8) ]
//   radial  G[l(j), n]   += exp(-eta (r_ij - Rs_n)^2) fc_r(r_ij)
//   angular G[p(j,k),m,n] += 2^(1-zeta) (1 + cos(theta_ijk - theta_m))^zeta
//                            exp(-eta ((r_ij + r_ik)/2 - Rs_n)^2) fc_a(r_ij) fc_a(r_ik)
//   fc(r) = 0.5 (cos(3.14159265359 r / Rc) + 1)
// cos(theta - theta_m) is formed as c cos(theta_m) + s sin(theta_m) with
// c = u_ij . u_ik and s = |u_ij x u_ik| >= 0, which is cos(acos(c) - theta_m)
// without the acos (and accurate for nearly collinear triples, where
// sqrt(1 - c^2) is not); the reference's clamp of c to +-(1 - 1e-16) only
// protects its acos and is a no-op in FP32.
//
// The adjoint takes dE/dG per atom (energy net + dE/dq * charge net), recomputes
// the pair/triple geometry from the positions, and produces
//   * the centre's own dE/dx_i,
//   * one scalar per radial edge and one vector per angular edge for the
//     neighbour side, gathered per atom through the reverse-edge index
//     (no atomics anywhere: the angular edge vectors are summed in one
//     shared-memory copy per 8-lane group, added in group order, so forces
//     are deterministic).
#include <cuda_runtime.h>

#include "tm_internal.h"

namespace {

struct DescArgs {
  const float4* xhi;
  const float4* xlo;
  const uint32_t* nbr_r;
  const uint32_t* nbr_a;
  const int32_t* cnt_r;
  const int32_t* cnt_a;
  const int32_t* rev_r;
  const int32_t* rev_a;
  const int32_t* row_of_atom;
  int N, KR, KA, Mpad;
  int prec;             // TM_PREC_FP32: hi/lo fp32 out; TM_PREC_BF16: bf16 out
  void* out0;
  void* out1;
  float* out_f32;       // optional plain fp32 rows [Mpad][Dp]
  float* gnorm2;        // optional squared L2 norm of each row [Mpad] (the relu
                        // refinement's error bound for the first layer)
  // adjoint
  const float* dEdG;    // [2*Mpad][Dp]
  const float* dEdq;    // [N]
  float4* fself;        // [N]
  float* sr;            // [N*KR]
  float4* va;           // [N*KA]
  float sh_hi[27][3];
  float sh_lo[27][3];
};

__device__ __forceinline__ void nbr_vec(const DescArgs& a, float4 hi, float4 lo, uint32_t e,
                                        float& dx, float& dy, float& dz, int& el) {
  const int j = (int)tm_atom(e);
  const int r = tm_img(e);
  const float4 hj = a.xhi[j], lj = a.xlo[j];
  dx = ds_sub_shift(hi.x, lo.x, hj.x, lj.x, a.sh_hi[r][0], a.sh_lo[r][0]);
  dy = ds_sub_shift(hi.y, lo.y, hj.y, lj.y, a.sh_hi[r][1], a.sh_lo[r][1]);
  dz = ds_sub_shift(hi.z, lo.z, hj.z, lj.z, a.sh_hi[r][2], a.sh_lo[r][2]);
  el = __float_as_int(hj.w);
}

// the neighbour vector as double-single components (hi + lo)
__device__ __forceinline__ void nbr_vec2(const DescArgs& a, float4 hi, float4 lo, uint32_t e,
                                         float (&dh)[3], float (&dl)[3], int& el) {
  const int j = (int)tm_atom(e);
  const int r = tm_img(e);
  const float4 hj = a.xhi[j], lj = a.xlo[j];
  ds_sub_shift2(hi.x, lo.x, hj.x, lj.x, a.sh_hi[r][0], a.sh_lo[r][0], dh[0], dl[0]);
  ds_sub_shift2(hi.y, lo.y, hj.y, lj.y, a.sh_hi[r][1], a.sh_lo[r][1], dh[1], dl[1]);
  ds_sub_shift2(hi.z, lo.z, hj.z, lj.z, a.sh_hi[r][2], a.sh_lo[r][2], dh[2], dl[2]);
  el = __float_as_int(hj.w);
}

// |d| of a double-single vector, as double-single
__device__ __forceinline__ void ds_norm(const float (&dh)[3], const float (&dl)[3], float& rh,
                                        float& rl) {
  float sh, sl, p, e, t;
  tm_two_prod(dh[0], dh[0], sh, sl);
  sl = fmaf(2.f * dh[0], dl[0], sl);
#pragma unroll
  for (int c = 1; c < 3; ++c) {
    tm_two_prod(dh[c], dh[c], p, e);
    tm_two_sum(sh, p, sh, t);
    sl += t + fmaf(2.f * dh[c], dl[c], e);
  }
  tm_fast_two_sum(sh, sl, sh, sl);
  tm_ds_sqrt(sh, sl, rh, rl);
}

// fc(r) = 0.5 (cos(pi_tf r / Rc) + 1) = sin^2(c (Rc - r)) for r = rh + rl,
// with c = c_hi + c_lo = pi_tf / (2 Rc): no cancellation near the cutoff and
// the argument carried to about 44 bits (sin^2(b + bl) ~ s^2 + 2 s cos(b) bl)
__device__ __forceinline__ float fcut_ds(float rh, float rl, float rc_hi, float rc_lo, float c_hi,
                                         float c_lo) {
  float dh, dl;
  tm_two_sum(rc_hi, -rh, dh, dl);
  dl += rc_lo - rl;
  float bh, bl;
  tm_two_prod(c_hi, dh, bh, bl);
  bl += fmaf(c_hi, dl, c_lo * dh);
  float sb, cb;
  sincosf(bh, &sb, &cb);
  return sb * fmaf(2.f * cb, bl, sb);
}

// (1 + c cos(th) + s sin(th))^8 for double-single c, s and constants, in
// double-single (squarings by exact products)
__device__ __forceinline__ float pow8_ds(float ch, float cl, float sh, float sl, float cth,
                                        float cth_lo, float sth, float sth_lo) {
  float p1, e1, p2, e2, th, tl;
  tm_two_prod(ch, cth, p1, e1);
  tm_two_prod(sh, sth, p2, e2);
  tm_two_sum(p1, p2, th, tl);
  tl += (e1 + e2) + (fmaf(ch, cth_lo, cl * cth) + fmaf(sh, sth_lo, sl * sth));
  float xh, xl;
  tm_two_sum(1.f, th, xh, xl);
  xl += tl;
  tm_fast_two_sum(xh, xl, xh, xl);
  if (xh <= 0.f) return 0.f;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    float ph, pl;
    tm_two_prod(xh, xh, ph, pl);
    pl = fmaf(2.f * xh, xl, pl);
    tm_fast_two_sum(ph, pl, xh, xl);
  }
  return xh + xl;
}

__device__ __forceinline__ float fcut(float r, float pi_tf, float rc) {
  return 0.5f * (cosf(pi_tf * r / rc) + 1.0f);
}
__device__ __forceinline__ float fcut_d(float r, float pi_tf, float rc) {
  return -0.5f * sinf(pi_tf * r / rc) * (pi_tf / rc);
}

// x^zeta for x >= 0 and its derivative factor zeta*x^(zeta-1)
__device__ __forceinline__ void powz(float x, const tm_consts& k, float& p, float& dp) {
  if (k.zeta_pow2) {  // zeta == 8
    const float x2 = x * x, x4 = x2 * x2, x7 = x4 * x2 * x;
    p = x7 * x;
    dp = 8.0f * x7;
  } else {
    p = powf(x, k.zeta);
    dp = k.zeta * powf(x, k.zeta - 1.0f);
  }
}

// Per-warp shared memory layout
struct WarpSmem {
  float* row;     // [Dp]
  float* ux;      // [KA]
  float* uy;
  float* uz;
  float* r;
  float* fc;
  float* fcd;
  float* vx;      // adjoint accumulators [KA]
  float* vy;
  float* vz;
};

__device__ __forceinline__ WarpSmem warp_smem(float* base, int Dp, int KA) {
  WarpSmem w;
  w.row = base;
  w.ux = base + Dp;
  w.uy = w.ux + KA;
  w.uz = w.uy + KA;
  w.r = w.uz + KA;
  w.fc = w.r + KA;
  w.fcd = w.fc + KA;
  w.vx = w.fcd + KA;
  w.vy = w.vx + KA;
  w.vz = w.vy + KA;
  return w;
}

__host__ __device__ __forceinline__ int smem_floats(int Dp, int KA) { return Dp + 9 * KA; }
// adjoint: the row, six geometry arrays and a [4 groups][3][KA] accumulator
__host__ __device__ __forceinline__ int smem_floats_adj(int Dp, int KA) { return Dp + 18 * KA; }

// angular neighbour geometry + element segments; returns segment starts in seg[]
__device__ __forceinline__ void load_angular(const DescArgs& a, const tm_consts& k, int i,
                                             float4 hi, float4 lo, int ca, WarpSmem& w,
                                             int* seg, int lane) {
  for (int e = 0; e <= k.nele; ++e) seg[e] = 0;
  for (int base = 0; base < ca; base += 32) {
    const int s = base + lane;
    int el = -1;
    if (s < ca) {
      float dx, dy, dz;
      nbr_vec(a, hi, lo, a.nbr_a[(size_t)i * a.KA + s], dx, dy, dz, el);
      const float r = sqrtf(dx * dx + dy * dy + dz * dz);
      const float inv = 1.0f / r;
      w.ux[s] = dx * inv;
      w.uy[s] = dy * inv;
      w.uz[s] = dz * inv;
      w.r[s] = r;
      w.fc[s] = fcut(r, k.pi_tf, k.a_rc);
      w.fcd[s] = fcut_d(r, k.pi_tf, k.a_rc);
    }
    // rows are sorted by element: count each element's neighbours by ballot
    for (int e = 0; e < k.nele; ++e) seg[e] += __popc(__ballot_sync(TM_FULL, el == e));
  }
  int acc = 0;
  for (int e = 0; e < k.nele; ++e) { int c = seg[e]; seg[e] = acc; acc += c; }
  seg[k.nele] = acc;
  __syncwarp();
}

// load_angular with double-single geometry (forward of the relu refinement):
// unit vectors hi in ux/uy/uz and lo in vx/vy/vz, |d| hi in r and lo in fcd,
// fc from the double-single distance
__device__ __forceinline__ void load_angular_ds(const DescArgs& a, const tm_consts& k, int i,
                                                float4 hi, float4 lo, int ca, WarpSmem& w,
                                                int* seg, int lane) {
  for (int e = 0; e <= k.nele; ++e) seg[e] = 0;
  for (int base = 0; base < ca; base += 32) {
    const int s = base + lane;
    int el = -1;
    if (s < ca) {
      float dh[3], dl[3], rh, rl;
      nbr_vec2(a, hi, lo, a.nbr_a[(size_t)i * a.KA + s], dh, dl, el);
      ds_norm(dh, dl, rh, rl);
      const float inv = __fdiv_rn(1.f, rh);
      float uh[3], ul[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        uh[c] = __fmul_rn(dh[c], inv);
        // (d - u r) / r with u = uh, r = rh + rl
        ul[c] = (fmaf(-uh[c], rh, dh[c]) + fmaf(-uh[c], rl, dl[c])) * inv;
      }
      w.ux[s] = uh[0]; w.uy[s] = uh[1]; w.uz[s] = uh[2];
      w.vx[s] = ul[0]; w.vy[s] = ul[1]; w.vz[s] = ul[2];
      w.r[s] = rh;
      w.fcd[s] = rl;
      w.fc[s] = fcut_ds(rh, rl, k.a_rc_hi, k.a_rc_lo, k.ca_hi, k.ca_lo);
    }
    for (int e = 0; e < k.nele; ++e) seg[e] += __popc(__ballot_sync(TM_FULL, el == e));
  }
  int acc = 0;
  for (int e = 0; e < k.nele; ++e) { int c = seg[e]; seg[e] = acc; acc += c; }
  seg[k.nele] = acc;
  __syncwarp();
}

// advance the (pa, pb) pair index by 4 in the enumeration order used for the
// element pair (b outer, a inner; a < b when both atoms share an element)
__device__ __forceinline__ void pair_advance(int& pa, int& pb, int na_, bool tri) {
  pa += 4;
  if (tri) {
    while (pa >= pb && pb > 0) { pa -= pb; ++pb; }
  } else {
    while (pa >= na_ && na_ > 0) { pa -= na_; ++pb; }
  }
}
// the same by `step` pairs
__device__ __forceinline__ void pair_advance_by(int& pa, int& pb, int na_, bool tri, int step) {
  pa += step;
  if (tri) {
    while (pa >= pb && pb > 0) { pa -= pb; ++pb; }
  } else {
    while (pa >= na_ && na_ > 0) { pa -= na_; ++pb; }
  }
}
__device__ __forceinline__ void pair_start(int t, int& pa, int& pb, int na_, bool tri) {
  if (tri) {
    int b = 1, acc = 0;
    while (acc + b <= t) { acc += b; ++b; }
    pb = b;
    pa = t - acc;
  } else {
    pb = na_ > 0 ? t / na_ : 0;
    pa = na_ > 0 ? t % na_ : 0;
  }
}

// ACC: the relu refinement's form, every difference vector, distance, cutoff
// function, angle term and Gaussian argument carried in double-single, so
// that each term is within a few FP32 roundings of its FP64 value (the plain
// form's FP32 distances put ~1e-7 relative error on the cutoff functions and
// the angle powers). Rows are still FP32 sums.
template <bool ACC>
__global__ void __launch_bounds__(128) k_desc_fwd(const DescArgs a, const tm_consts k) {
  extern __shared__ float sh[];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + wib;
  if (i >= a.N) return;
  WarpSmem w = warp_smem(sh + (size_t)wib * smem_floats(k.Dp, a.KA), k.Dp, a.KA);
  for (int c = lane; c < k.Dp; c += 32) w.row[c] = 0.f;
  __syncwarp();
  const float4 hi = a.xhi[i], lo = a.xlo[i];
  // ---- radial ----
  const int cr = a.cnt_r[i];
  const float rs_lane = k.rs_r[lane < k.nr ? lane : 0];
  const float rs_lane_lo = k.rs_r_lo[lane < k.nr ? lane : 0];
  float racc = 0.f;
  int rel = -1;
  for (int base = 0; base < cr; base += 32) {
    const int s = base + lane;
    float r = 0.f, rl = 0.f, f = 0.f;
    int el = 0;
    if (s < cr) {
      if constexpr (ACC) {
        float dh[3], dl[3];
        nbr_vec2(a, hi, lo, a.nbr_r[(size_t)i * a.KR + s], dh, dl, el);
        ds_norm(dh, dl, r, rl);
        f = fcut_ds(r, rl, k.r_rc_hi, k.r_rc_lo, k.cr_hi, k.cr_lo);
      } else {
        float dx, dy, dz;
        nbr_vec(a, hi, lo, a.nbr_r[(size_t)i * a.KR + s], dx, dy, dz, el);
        r = sqrtf(dx * dx + dy * dy + dz * dz);
        f = fcut(r, k.pi_tf, k.r_rc);
      }
    }
    // rows are sorted by element: accumulate in a register, flush to the
    // row when the element changes (at most nele flushes per centre)
    const int n = min(32, cr - base);
    for (int q = 0; q < n; ++q) {
      const float rq = __shfl_sync(TM_FULL, r, q);
      const float fq = __shfl_sync(TM_FULL, f, q);
      const int lq = __shfl_sync(TM_FULL, el, q);
      if (lq != rel) {
        if (rel >= 0 && lane < k.nr) w.row[rel * k.nr + lane] += racc;
        racc = 0.f;
        rel = lq;
      }
      float t;
      if constexpr (ACC) {
        const float rlq = __shfl_sync(TM_FULL, rl, q);
        t = __fadd_rn(__fsub_rn(rq, rs_lane), __fsub_rn(rlq, rs_lane_lo));
      } else {
        t = rq - rs_lane;
      }
      racc += expf(-k.eta * t * t) * fq;
    }
  }
  if (rel >= 0 && lane < k.nr) w.row[rel * k.nr + lane] += racc;
  // ---- angular ----
  const int ca = a.cnt_a[i];
  int seg[TM_MAX_ELE + 1];
  if constexpr (ACC) load_angular_ds(a, k, i, hi, lo, ca, w, seg, lane);
  else load_angular(a, k, i, hi, lo, ca, w, seg, lane);
  const int grp = lane >> 3, q = lane & 7;
  const float cth = k.cos_th[q], sth = k.sin_th[q], rsq = k.rs_a[q];
  const float cth_lo = k.cos_th_lo[q], sth_lo = k.sin_th_lo[q], rsq_lo = k.rs_a_lo[q];
  for (int ea = 0; ea < k.nele; ++ea) {
    for (int eb = ea; eb < k.nele; ++eb) {
      const int na_ = seg[ea + 1] - seg[ea], nb_ = seg[eb + 1] - seg[eb];
      const bool tri = (ea == eb);
      const int npair = tri ? na_ * (na_ - 1) / 2 : na_ * nb_;
      if (npair == 0) continue;
      const int l = k.elepair[ea][eb];
      float acc[8];
#pragma unroll
      for (int n = 0; n < 8; ++n) acc[n] = 0.f;
      if constexpr (ACC) {
        // The double-single quantities of a triple that do not depend on the
        // angle bin or shell (cos and sin of the angle, the cutoff factors,
        // the mean distance) are computed once, by one lane per triple for 32
        // triples a round; each group of 8 lanes then takes its triples' values
        // by shuffle (the same triples in the same order as below, so the
        // rows are the same bit for bit).
        int pa, pb;
        pair_start(lane, pa, pb, na_, tri);
        for (int tb = 0; tb < npair; tb += 32) {
          float tch = 0.f, tcl = 0.f, tsh = 0.f, tsl = 0.f, tfa = 0.f, tfb = 0.f, trh = 0.f, trl = 0.f;
          if (tb + lane < npair) {
            const int sa = seg[ea] + pa, sb = seg[eb] + pb;
            // c = u_a . u_b and s = sqrt((1 - c)(1 + c)) in double-single (c is
            // accurate to ~2^-44, so s is accurate even for nearly collinear triples)
            float ch, cl, p, e, t;
            tm_two_prod(w.ux[sa], w.ux[sb], ch, cl);
            cl += fmaf(w.ux[sa], w.vx[sb], w.vx[sa] * w.ux[sb]);
            tm_two_prod(w.uy[sa], w.uy[sb], p, e);
            tm_two_sum(ch, p, ch, t);
            cl += t + e + fmaf(w.uy[sa], w.vy[sb], w.vy[sa] * w.uy[sb]);
            tm_two_prod(w.uz[sa], w.uz[sb], p, e);
            tm_two_sum(ch, p, ch, t);
            cl += t + e + fmaf(w.uz[sa], w.vz[sb], w.vz[sa] * w.uz[sb]);
            tm_fast_two_sum(ch, cl, ch, cl);
            float mh, ml, ph, pl, qh, ql;
            tm_two_sum(1.f, -ch, mh, ml);
            ml -= cl;
            tm_two_sum(1.f, ch, ph, pl);
            pl += cl;
            tm_two_prod(mh, ph, qh, ql);
            ql += fmaf(mh, pl, ml * ph);
            tm_fast_two_sum(qh, ql, qh, ql);
            tm_ds_sqrt(qh, ql, tsh, tsl);
            tch = ch;
            tcl = cl;
            tfa = w.fc[sa];
            tfb = w.fc[sb];
            // r_a + r_b in double-single
            tm_two_sum(w.r[sa], w.r[sb], trh, trl);
            trl += w.fcd[sa] + w.fcd[sb];
          }
          pair_advance_by(pa, pb, na_, tri, 32);
          const int nt = min(32, npair - tb);
          for (int j0 = 0; j0 < nt; j0 += 8) {
            float AF[2], B[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int src = j0 + 4 * h + grp;
              const float ch = __shfl_sync(TM_FULL, tch, src), cl = __shfl_sync(TM_FULL, tcl, src);
              const float sh = __shfl_sync(TM_FULL, tsh, src), sl = __shfl_sync(TM_FULL, tsl, src);
              const float fa = __shfl_sync(TM_FULL, tfa, src), fb = __shfl_sync(TM_FULL, tfb, src);
              const float rh = __shfl_sync(TM_FULL, trh, src), rl2 = __shfl_sync(TM_FULL, trl, src);
              AF[h] = 0.f;
              B[h] = 0.f;
              if (src < nt) {
                float pw;
                if (k.zeta_pow2) {
                  pw = pow8_ds(ch, cl, sh, sl, cth, cth_lo, sth, sth_lo);
                } else {
                  float dp;
                  powz(fmaxf(0.f, 1.f + (ch * cth + sh * sth)), k, pw, dp);
                }
                AF[h] = k.two_1mz * pw * fa * fb;
                // (r_a + r_b) / 2 - Rs in double-single
                const float u = __fadd_rn(__fsub_rn(0.5f * rh, rsq), __fsub_rn(0.5f * rl2, rsq_lo));
                B[h] = expf(-k.eta * u * u);
              }
            }
#pragma unroll
            for (int n = 0; n < 8; ++n) {
              const float B0 = __shfl_sync(TM_FULL, B[0], (lane & ~7) | n);
              const float B1 = __shfl_sync(TM_FULL, B[1], (lane & ~7) | n);
              acc[n] += AF[0] * B0 + AF[1] * B1;
            }
          }
        }
      } else {
        int pa, pb;
        pair_start(grp, pa, pb, na_, tri);
        // FP32 form: two triples per group per iteration (independent chains
        // for latency)
        for (int tb = 0; tb < npair; tb += 8) {
          float AF[2], B[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            AF[h] = 0.f;
            B[h] = 0.f;
            if (tb + 4 * h + grp < npair) {
              const int sa = seg[ea] + pa, sb = seg[eb] + pb;
              const float c = w.ux[sa] * w.ux[sb] + w.uy[sa] * w.uy[sb] + w.uz[sa] * w.uz[sb];
              // sin(theta) = |u_a x u_b|: well conditioned for nearly collinear triples,
              // where sqrt(1 - c^2) loses most of its digits in FP32
              const float nx = w.uy[sa] * w.uz[sb] - w.uz[sa] * w.uy[sb];
              const float ny = w.uz[sa] * w.ux[sb] - w.ux[sa] * w.uz[sb];
              const float nz = w.ux[sa] * w.uy[sb] - w.uy[sa] * w.ux[sb];
              const float sn = sqrtf(nx * nx + ny * ny + nz * nz);
              const float T = c * cth + sn * sth;
              float p, dp;
              powz(fmaxf(0.f, 1.f + T), k, p, dp);
              AF[h] = k.two_1mz * p * w.fc[sa] * w.fc[sb];
              const float u = 0.5f * (w.r[sa] + w.r[sb]) - rsq;
              B[h] = expf(-k.eta * u * u);
            }
            pair_advance(pa, pb, na_, tri);
          }
#pragma unroll
          for (int n = 0; n < 8; ++n) {
            const float B0 = __shfl_sync(TM_FULL, B[0], (lane & ~7) | n);
            const float B1 = __shfl_sync(TM_FULL, B[1], (lane & ~7) | n);
            acc[n] += AF[0] * B0 + AF[1] * B1;
          }
        }
      }
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        acc[n] += __shfl_xor_sync(TM_FULL, acc[n], 8);
        acc[n] += __shfl_xor_sync(TM_FULL, acc[n], 16);
      }
      if (grp == 0) {
        float* dst = w.row + k.nele * k.nr + l * 64 + q * 8;
#pragma unroll
        for (int n = 0; n < 8; ++n) dst[n] = acc[n];
      }
    }
  }
  __syncwarp();
  // ---- write the row (element-sorted order) ----
  const int row = a.row_of_atom[i];
  if (a.prec == TM_PREC_FP32) {
    float4* o0 = reinterpret_cast<float4*>(static_cast<float*>(a.out0) + (size_t)row * k.Dp);
    float4* o1 = reinterpret_cast<float4*>(static_cast<float*>(a.out1) + (size_t)row * k.Dp);
    for (int c = lane; c < k.Dp / 4; c += 32) {
      float4 v = reinterpret_cast<const float4*>(w.row)[c];
      float4 h, l;
      tm_tf32_split(v.x, h.x, l.x);
      tm_tf32_split(v.y, h.y, l.y);
      tm_tf32_split(v.z, h.z, l.z);
      tm_tf32_split(v.w, h.w, l.w);
      o0[c] = h;
      o1[c] = l;
    }
  } else {
    uint2* o0 = reinterpret_cast<uint2*>(static_cast<uint16_t*>(a.out0) + (size_t)row * k.Dp);
    for (int c = lane; c < k.Dp / 4; c += 32) {
      float4 v = reinterpret_cast<const float4*>(w.row)[c];
      __nv_bfloat162 p0 = __floats2bfloat162_rn(v.x, v.y);
      __nv_bfloat162 p1 = __floats2bfloat162_rn(v.z, v.w);
      o0[c] = make_uint2(*reinterpret_cast<uint32_t*>(&p0), *reinterpret_cast<uint32_t*>(&p1));
    }
  }
  if (a.out_f32) {
    float4* o = reinterpret_cast<float4*>(a.out_f32 + (size_t)row * k.Dp);
    for (int c = lane; c < k.Dp / 4; c += 32) o[c] = reinterpret_cast<const float4*>(w.row)[c];
  }
  if (a.gnorm2) {
    float ss = 0.f;
    for (int c = lane; c < k.Dp / 4; c += 32) {
      const float4 v = reinterpret_cast<const float4*>(w.row)[c];
      ss += v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w;
    }
    ss = warp_sum(ss);
    if (lane == 0) a.gnorm2[row] = ss;
  }
}

__global__ void __launch_bounds__(128, 6) k_desc_adj(const DescArgs a, const tm_consts k) {
  extern __shared__ float sh[];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + wib;
  if (i >= a.N) return;
  WarpSmem w = warp_smem(sh + (size_t)wib * smem_floats_adj(k.Dp, a.KA), k.Dp, a.KA);
  // neighbour-side angular gradients: one copy per 8-lane group, so that no
  // two lanes of an instruction update the same word (no atomics); the copies
  // are added in group order at the end
  float* vacc = w.fcd + a.KA;
  // upstream dE/dG for this centre: energy net + dE/dq * charge net
  const int row = a.row_of_atom[i];
  const float dq = a.dEdq[i];
  const float* gE = a.dEdG + (size_t)row * k.Dp;
  const float* gQ = a.dEdG + ((size_t)a.Mpad + row) * k.Dp;
  for (int c = lane; c < k.Dp; c += 32) w.row[c] = gE[c] + dq * gQ[c];
  __syncwarp();
  const float4 hi = a.xhi[i], lo = a.xlo[i];
  float fx = 0.f, fy = 0.f, fz = 0.f;   // dE/dx_i, per-lane partials
  // ---- radial ----
  const int cr = a.cnt_r[i];
  for (int base = 0; base < cr; base += 32) {
    const int s = base + lane;
    float r = 1.f, f = 0.f, fd = 0.f, dx = 0.f, dy = 0.f, dz = 0.f;
    int el = 0;
    if (s < cr) {
      nbr_vec(a, hi, lo, a.nbr_r[(size_t)i * a.KR + s], dx, dy, dz, el);
      r = sqrtf(dx * dx + dy * dy + dz * dz);
      f = fcut(r, k.pi_tf, k.r_rc);
      fd = fcut_d(r, k.pi_tf, k.r_rc);
    }
    // lane = edge: S = sum_n dE/dG[l, n] d/dr (exp(-eta (r - Rs_n)^2) fc(r)),
    // the row read from shared memory as broadcasts within each element
    float myS = 0.f;
    if (s < cr) {
      const float* up = w.row + el * k.nr;
      for (int n = 0; n < k.nr; ++n) {
        const float t = r - k.rs_r[n];
        const float g = expf(-k.eta * t * t);
        myS += up[n] * g * (-2.f * k.eta * t * f + fd);
      }
    }
    if (s < cr) {
      a.sr[(size_t)i * a.KR + s] = myS;
      const float inv = 1.f / r;
      fx += myS * dx * inv;
      fy += myS * dy * inv;
      fz += myS * dz * inv;
    }
  }
  // ---- angular ----
  const int ca = a.cnt_a[i];
  int seg[TM_MAX_ELE + 1];
  load_angular(a, k, i, hi, lo, ca, w, seg, lane);
  for (int s = lane; s < 12 * a.KA; s += 32) vacc[s] = 0.f;
  __syncwarp();
  const int grp = lane >> 3, q = lane & 7;
  const float cth = k.cos_th[q], sth = k.sin_th[q], rsq = k.rs_a[q];
  float fown = 0.f;   // lanes q = 0..5: one component of the centre's angular dE/dx
  for (int ea = 0; ea < k.nele; ++ea) {
    for (int eb = ea; eb < k.nele; ++eb) {
      const int na_ = seg[ea + 1] - seg[ea], nb_ = seg[eb + 1] - seg[eb];
      const bool tri = (ea == eb);
      const int npair = tri ? na_ * (na_ - 1) / 2 : na_ * nb_;
      if (npair == 0) continue;
      const int l = k.elepair[ea][eb];
      float wl[8];
      const float* src = w.row + k.nele * k.nr + l * 64 + q * 8;
#pragma unroll
      for (int n = 0; n < 8; ++n) wl[n] = src[n];
      int pa, pb;
      pair_start(grp, pa, pb, na_, tri);
      // two triples per group per iteration; the six output components of a
      // triple (a-side xyz, b-side xyz) go to lanes q = 0..5 of its group
      for (int tb = 0; tb < npair; tb += 8) {
        int sa[2], sb[2];
        bool act[2];
        float sn[2], A[2], dA[2], B[2], Bd[2], nx[2], ny[2], nz[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          act[h] = tb + 4 * h + grp < npair;
          sa[h] = 0; sb[h] = 0;
          sn[h] = 0.f; A[h] = 0.f; dA[h] = 0.f; B[h] = 0.f; Bd[h] = 0.f;
          nx[h] = 0.f; ny[h] = 0.f; nz[h] = 0.f;
          if (act[h]) {
            const int ia = seg[ea] + pa, ib = seg[eb] + pb;
            sa[h] = ia;
            sb[h] = ib;
            const float c = w.ux[ia] * w.ux[ib] + w.uy[ia] * w.uy[ib] + w.uz[ia] * w.uz[ib];
            // n = u_a x u_b, sin(theta) = |n| (accurate near collinearity)
            nx[h] = w.uy[ia] * w.uz[ib] - w.uz[ia] * w.uy[ib];
            ny[h] = w.uz[ia] * w.ux[ib] - w.ux[ia] * w.uz[ib];
            nz[h] = w.ux[ia] * w.uy[ib] - w.uy[ia] * w.ux[ib];
            sn[h] = sqrtf(nx[h] * nx[h] + ny[h] * ny[h] + nz[h] * nz[h]);
            const float T = c * cth + sn[h] * sth;
            const float dT = -(sn[h] * cth - c * sth);   // d cos(theta - theta_m) / d theta
            float p, dp;
            powz(fmaxf(0.f, 1.f + T), k, p, dp);
            A[h] = k.two_1mz * p;
            dA[h] = k.two_1mz * dp * dT;
            const float u = 0.5f * (w.r[ia] + w.r[ib]) - rsq;
            B[h] = expf(-k.eta * u * u);
            Bd[h] = B[h] * (-2.f * k.eta * u);
          }
          pair_advance(pa, pb, na_, tri);
        }
        float P[2] = {0.f, 0.f}, Q[2] = {0.f, 0.f};
#pragma unroll
        for (int n = 0; n < 8; ++n) {
          const int src_lane = (lane & ~7) | n;
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            P[h] += wl[n] * __shfl_sync(TM_FULL, B[h], src_lane);
            Q[h] += wl[n] * __shfl_sync(TM_FULL, Bd[h], src_lane);
          }
        }
        float S1[2], S2[2], S3[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          S1[h] = A[h] * P[h];
          S2[h] = A[h] * Q[h];
          S3[h] = dA[h] * P[h];
        }
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            S1[h] += __shfl_xor_sync(TM_FULL, S1[h], o);
            S2[h] += __shfl_xor_sync(TM_FULL, S2[h], o);
            S3[h] += __shfl_xor_sync(TM_FULL, S3[h], o);
          }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (act[h] && q < 6) {
            const int ia = sa[h], ib = sb[h];
            const float fa = w.fc[ia], fb = w.fc[ib];
            const float fcc = fa * fb;
            const bool bside = q >= 3;
            const int d = bside ? q - 3 : q;
            // dE/dr along the edge, and d theta / d d = -(u_o - c u) / (r sin theta):
            // the in-plane directions are n x u_a and u_b x n, of length sin theta
            const float dr = 0.5f * S2[h] * fcc + S1[h] * (bside ? fa * w.fcd[ib] : w.fcd[ia] * fb);
            const float kc = -(S3[h] * fcc) / fmaxf(sn[h], 1e-30f);
            const int e = bside ? ib : ia;
            const float* U0 = d == 0 ? w.ux : (d == 1 ? w.uy : w.uz);
            const float* U1 = d == 0 ? w.uy : (d == 1 ? w.uz : w.ux);
            const float* U2 = d == 0 ? w.uz : (d == 1 ? w.ux : w.uy);
            const float n1 = d == 0 ? ny[h] : (d == 1 ? nz[h] : nx[h]);
            const float n2 = d == 0 ? nz[h] : (d == 1 ? nx[h] : ny[h]);
            // a side: (n x u_a)_d = n1 u2 - n2 u1; b side: (u_b x n)_d = u1 n2 - u2 n1
            const float perp = bside ? (U1[e] * n2 - U2[e] * n1) : (n1 * U2[e] - n2 * U1[e]);
            const float g = dr * U0[e] + (kc / w.r[e]) * perp;
            fown += g;
            vacc[(grp * 3 + d) * a.KA + e] -= g;
          }
        }
        __syncwarp();
      }
    }
  }
  __syncwarp();
  for (int s = lane; s < ca; s += 32) {
    float v[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      v[d] = ((vacc[d * a.KA + s] + vacc[(3 + d) * a.KA + s]) + vacc[(6 + d) * a.KA + s]) +
             vacc[(9 + d) * a.KA + s];
    a.va[(size_t)i * a.KA + s] = make_float4(v[0], v[1], v[2], 0.f);
  }
  fx += (q == 0 || q == 3) ? fown : 0.f;
  fy += (q == 1 || q == 4) ? fown : 0.f;
  fz += (q == 2 || q == 5) ? fown : 0.f;
  fx = warp_sum(fx);
  fy = warp_sum(fy);
  fz = warp_sum(fz);
  if (lane == 0) a.fself[i] = make_float4(fx, fy, fz, 0.f);
}

}  // namespace

// shared helpers used by tm_api.cu
void tm_fill_shifts(const tm_system* s, float hi[27][3], float lo[27][3]) {
  for (int r = 0; r < 27; ++r) {
    const int sx = r / 9 - 1, sy = (r / 3) % 3 - 1, sz = r % 3 - 1;
    for (int d = 0; d < 3; ++d) {
      double v = 0.0;
      if (s->periodic) v = sx * s->lat[0 + d] + sy * s->lat[3 + d] + sz * s->lat[6 + d];
      const float h = (float)v;
      hi[r][d] = h;
      lo[r][d] = (float)(v - (double)h);
    }
  }
}

static DescArgs make_desc_args(tm_system* s) {
  DescArgs a;
  a.xhi = s->d_xhi; a.xlo = s->d_xlo; a.nbr_r = s->d_nbr_r; a.nbr_a = s->d_nbr_a;
  a.cnt_r = s->d_cnt_r; a.cnt_a = s->d_cnt_a; a.rev_r = s->d_rev_r; a.rev_a = s->d_rev_a;
  a.row_of_atom = s->row_of_atom; a.N = s->N; a.KR = s->KR; a.KA = s->KA; a.Mpad = s->Mpad;
  a.prec = s->model->desc.precision;
  a.out0 = s->G[0]; a.out1 = s->G[1]; a.out_f32 = nullptr; a.gnorm2 = s->kink_g2;
  a.dEdG = s->dEdG; a.dEdq = s->d_dEdq; a.fself = s->d_fself; a.sr = s->d_sr; a.va = s->d_va;
  tm_fill_shifts(s, a.sh_hi, a.sh_lo);
  return a;
}

static int launch_desc_fwd(tm_system* s, const DescArgs& a) {
  tm_ctx* ctx = s->ctx;
  const tm_consts& k = s->model->k;
  const size_t shm = (size_t)4 * smem_floats(k.Dp, s->KA) * sizeof(float);
  // the double-single form for the relu refinement (tm_gemm.cu)
  const bool acc = s->model->kink;
  if (shm > 48 * 1024)
    cudaFuncSetAttribute(acc ? k_desc_fwd<true> : k_desc_fwd<false>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (acc) k_desc_fwd<true><<<tm_div_up(s->N, 4), 128, shm, ctx->stream>>>(a, k);
  else k_desc_fwd<false><<<tm_div_up(s->N, 4), 128, shm, ctx->stream>>>(a, k);
  ctx->launches++;
  return tm_cuda_check(ctx, cudaGetLastError(), "descriptors");
}

int tm_launch_descriptors(tm_system* s) { return launch_desc_fwd(s, make_desc_args(s)); }

int tm_launch_descriptors_f32(tm_system* s, float* out) {
  DescArgs a = make_desc_args(s);
  a.out_f32 = out;
  return launch_desc_fwd(s, a);
}

namespace {
struct GatherArgs {
  const float4* xhi;
  const float4* xlo;
  const uint32_t* nbr_r;
  const uint32_t* nbr_a;
  const int32_t* cnt_r;
  const int32_t* cnt_a;
  const int32_t* rev_r;
  const int32_t* rev_a;
  const float4* fself;
  const float* sr;
  const float4* va;
  const float4* fcv;
  double* F;
  int N, KR, KA;
  int ref_periodic;   // drop neighbour-side terms that reach an atom through an image
  double scale;       // -JOULEPERHARTREE
  float sh_hi[27][3];
  float sh_lo[27][3];
};

__global__ void __launch_bounds__(128) k_force_gather(const GatherArgs a) {
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + wib;
  if (i >= a.N) return;
  const float4 hi = a.xhi[i], lo = a.xlo[i];
  float gx = 0.f, gy = 0.f, gz = 0.f;
  const int cr = a.cnt_r[i];
  for (int s = lane; s < cr; s += 32) {
    const uint32_t e = a.nbr_r[(size_t)i * a.KR + s];
    const int rv = a.rev_r[(size_t)i * a.KR + s];
    if (rv < 0) continue;
    if (a.ref_periodic && tm_img(e) != TM_IMG_SELF) continue;
    const int j = (int)tm_atom(e), r = tm_img(e);
    const float4 hj = a.xhi[j], lj = a.xlo[j];
    const float dx = ds_sub_shift(hi.x, lo.x, hj.x, lj.x, a.sh_hi[r][0], a.sh_lo[r][0]);
    const float dy = ds_sub_shift(hi.y, lo.y, hj.y, lj.y, a.sh_hi[r][1], a.sh_lo[r][1]);
    const float dz = ds_sub_shift(hi.z, lo.z, hj.z, lj.z, a.sh_hi[r][2], a.sh_lo[r][2]);
    const float S = a.sr[rv] / sqrtf(dx * dx + dy * dy + dz * dz);
    gx += S * dx;
    gy += S * dy;
    gz += S * dz;
  }
  const int ca = a.cnt_a[i];
  for (int s = lane; s < ca; s += 32) {
    const uint32_t e = a.nbr_a[(size_t)i * a.KA + s];
    const int rv = a.rev_a[(size_t)i * a.KA + s];
    if (rv < 0) continue;
    if (a.ref_periodic && tm_img(e) != TM_IMG_SELF) continue;
    const float4 v = a.va[rv];
    gx += v.x;
    gy += v.y;
    gz += v.z;
  }
  gx = warp_sum(gx);
  gy = warp_sum(gy);
  gz = warp_sum(gz);
  if (lane == 0) {
    const float4 f0 = a.fself[i];
    const float4 fc = a.fcv[i];
    a.F[3 * i + 0] = a.scale * ((double)f0.x + (double)gx + (double)fc.x);
    a.F[3 * i + 1] = a.scale * ((double)f0.y + (double)gy + (double)fc.y);
    a.F[3 * i + 2] = a.scale * ((double)f0.z + (double)gz + (double)fc.z);
  }
}
}  // namespace

int tm_launch_adjoint(tm_system* s, unsigned flags) {
  tm_ctx* ctx = s->ctx;
  DescArgs a = make_desc_args(s);
  const tm_consts& k = s->model->k;
  const size_t shm = (size_t)4 * smem_floats_adj(k.Dp, s->KA) * sizeof(float);
  if (shm > 48 * 1024)
    cudaFuncSetAttribute(k_desc_adj, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  k_desc_adj<<<tm_div_up(s->N, 4), 128, shm, ctx->stream>>>(a, k);
  GatherArgs g;
  g.xhi = s->d_xhi; g.xlo = s->d_xlo; g.nbr_r = s->d_nbr_r; g.nbr_a = s->d_nbr_a;
  g.cnt_r = s->d_cnt_r; g.cnt_a = s->d_cnt_a; g.rev_r = s->d_rev_r; g.rev_a = s->d_rev_a;
  g.fself = s->d_fself; g.sr = s->d_sr; g.va = s->d_va; g.fcv = s->d_fcv; g.F = s->d_F;
  g.N = s->N; g.KR = s->KR; g.KA = s->KA;
  g.ref_periodic = (s->periodic && (flags & TM_F_REFERENCE_PERIODIC_FORCE)) ? 1 : 0;
  g.scale = -2625.499638 * 1000.0;   // -JOULEPERHARTREE (PhysicalData.py:36-37)
  tm_fill_shifts(s, g.sh_hi, g.sh_lo);
  k_force_gather<<<tm_div_up(s->N, 4), 128, 0, ctx->stream>>>(g);
  ctx->launches += 2;
  return tm_cuda_check(ctx, cudaGetLastError(), "adjoint");
}
