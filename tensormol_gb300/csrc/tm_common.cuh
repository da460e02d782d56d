// Shared device helpers for the BP+EE energy/force kernels (sm_103a).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/tmgpu.h"

#define TM_WARP 32
#define TM_FULL 0xffffffffu

// Device status word written by kernels: first error wins.
struct tm_dev_status {
  int code;     // TM_OK or TM_E_*
  int detail;   // kernel-specific (index, needed capacity, ...)
  int where;    // kernel id
  int pad;
};

__device__ __forceinline__ void tm_flag(tm_dev_status* st, int code, int detail, int where) {
  if (atomicCAS(&st->code, 0, code) == 0) {
    st->detail = detail;
    st->where = where;
  }
}

// ---------------------------------------------------------------------------
// Double-single positions: x = hi + lo with hi = fp32(x), lo = fp32(x - hi).
// The difference of two such positions is accurate to about one fp32 ulp of
// the *difference*, independent of the coordinates' magnitude.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float ds_sub(float ahi, float alo, float bhi, float blo) {
  // TwoSum on the hi parts keeps the rounding error of (ahi - bhi).
  float s = __fsub_rn(ahi, bhi);
  float bb = __fsub_rn(s, ahi);
  float err = __fadd_rn(__fsub_rn(ahi, __fsub_rn(s, bb)), __fsub_rn(-bhi, bb));
  return __fadd_rn(s, __fadd_rn(err, __fsub_rn(alo, blo)));
}

// Same with an image shift (shi, slo) added to b.
__device__ __forceinline__ float ds_sub_shift(float ahi, float alo, float bhi, float blo,
                                              float shi, float slo) {
  float s = __fsub_rn(ahi, bhi);
  float bb = __fsub_rn(s, ahi);
  float err = __fadd_rn(__fsub_rn(ahi, __fsub_rn(s, bb)), __fsub_rn(-bhi, bb));
  // s - shi: both of similar magnitude when the image is the near one
  float t = __fsub_rn(s, shi);
  float tb = __fsub_rn(t, s);
  float err2 = __fadd_rn(__fsub_rn(s, __fsub_rn(t, tb)), __fsub_rn(-shi, tb));
  return __fadd_rn(t, __fadd_rn(__fadd_rn(err, err2), __fsub_rn(__fsub_rn(alo, blo), slo)));
}

// Same, keeping the result as an unevaluated sum hi + lo (about 44 bits).
__device__ __forceinline__ void ds_sub_shift2(float ahi, float alo, float bhi, float blo, float shi,
                                              float slo, float& hi, float& lo) {
  float s = __fsub_rn(ahi, bhi);
  float bb = __fsub_rn(s, ahi);
  float err = __fadd_rn(__fsub_rn(ahi, __fsub_rn(s, bb)), __fsub_rn(-bhi, bb));
  float t = __fsub_rn(s, shi);
  float tb = __fsub_rn(t, s);
  float err2 = __fadd_rn(__fsub_rn(s, __fsub_rn(t, tb)), __fsub_rn(-shi, tb));
  const float c = __fadd_rn(__fadd_rn(err, err2), __fsub_rn(__fsub_rn(alo, blo), slo));
  hi = __fadd_rn(t, c);
  lo = __fsub_rn(c, __fsub_rn(hi, t));
}

// ---------------------------------------------------------------------------
// Error-free transformations for double-single (hi + lo) arithmetic: Knuth's
// TwoSum, Dekker's FastTwoSum (|a| >= |b|) and the FMA form of TwoProduct.
// The _rn intrinsics keep the compiler from contracting them into FMAs.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tm_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void tm_fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ void tm_two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}
// sqrt of a double-single s = sh + sl >= 0 (one Newton correction)
__device__ __forceinline__ void tm_ds_sqrt(float sh, float sl, float& rh, float& rl) {
  if (sh <= 0.f) { rh = 0.f; rl = 0.f; return; }
  rh = sqrtf(sh);
  rl = __fmul_rn(__fadd_rn(__fmaf_rn(-rh, rh, sh), sl), __fdiv_rn(0.5f, rh));
}

// ---------------------------------------------------------------------------
// The reference's membership test, C_API/MolEmb.cpp:1214-1218:
//   dij = sqrt(dx*dx + dy*dy + dz*dz) + 1e-13;  accept if dij < rng
// in IEEE double with each operation rounded separately (no contraction).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool tm_exact_within(double xi, double yi, double zi, double xj,
                                                double yj, double zj, double rng) {
  double dx = __dsub_rn(xi, xj);
  double dy = __dsub_rn(yi, yj);
  double dz = __dsub_rn(zi, zj);
  double s = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  s = __dadd_rn(s, __dmul_rn(dz, dz));
  double d = __dadd_rn(__dsqrt_rn(s), 0.0000000000001);
  return d < rng;
}

// Image coordinate x + i*a0 + j*a1 + k*a2 formed left to right as the
// reference's tessellation does (ForceModifiers/Periodic.py:170-173).
__device__ __forceinline__ double tm_image_coord(double x, int i, int j, int k, double a0,
                                                 double a1, double a2) {
  double v = __dadd_rn(x, __dmul_rn((double)i, a0));
  v = __dadd_rn(v, __dmul_rn((double)j, a1));
  v = __dadd_rn(v, __dmul_rn((double)k, a2));
  return v;
}

// Image code of a neighbour entry: raster index r = 9(i+1) + 3(j+1) + (k+1)
// over shifts (i,j,k) in {-1,0,1}^3; r = 13 is the cell itself. Entries are
// packed as (r << 27) | atom, atom < 2^27.
#define TM_IMG_SHIFT 27
#define TM_ATOM_MASK ((1u << TM_IMG_SHIFT) - 1u)
#define TM_IMG_SELF 13

__device__ __forceinline__ uint32_t tm_pack(uint32_t atom, int r) {
  return ((uint32_t)r << TM_IMG_SHIFT) | atom;
}
__device__ __forceinline__ uint32_t tm_atom(uint32_t e) { return e & TM_ATOM_MASK; }
__device__ __forceinline__ int tm_img(uint32_t e) { return (int)(e >> TM_IMG_SHIFT); }
// Index of an image in the reference's tessellated ordering
// (Periodic.py:158-173): 0 = real, then raster order skipping (0,0,0).
__device__ __forceinline__ int tm_ref_image_index(int r) {
  return r == TM_IMG_SELF ? 0 : (r < TM_IMG_SELF ? r + 1 : r);
}
__device__ __forceinline__ void tm_img_ijk(int r, int& i, int& j, int& k) {
  i = r / 9 - 1;
  j = (r / 3) % 3 - 1;
  k = r % 3 - 1;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(TM_FULL, v, o);
  return v;
}

// Split of an FP32 value into two TF32 values for the 3-pass tensor-core
// product: hi = x rounded to nearest TF32 (10 mantissa bits; add half an ulp
// of the kept bits, clear the 13 low bits), lo = x - hi (exact in FP32) rounded
// the same way. Rounding to nearest (rather than truncating) keeps both parts'
// errors unbiased; |x - hi - lo| <= 2^-23 |x|.
__host__ __device__ __forceinline__ float tm_tf32_rn(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  u = (u + 0x1000u) & 0xffffe000u;
  float r;
  memcpy(&r, &u, 4);
  return r;
}
__host__ __device__ __forceinline__ void tm_tf32_split(float x, float& hi, float& lo) {
  hi = tm_tf32_rn(x);
  lo = tm_tf32_rn(x - hi);
}
