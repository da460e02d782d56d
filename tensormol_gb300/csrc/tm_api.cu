// C ABI entry points: context, model, system, energy/force, neighbour export.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>

#include <cmath>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "tm_internal.h"

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
int tm_fail(tm_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int tm_cuda_check(tm_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return TM_OK;
  return tm_fail(ctx, TM_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int tm_alloc(tm_ctx* ctx, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  if (ctx->budget && ctx->in_use + bytes > ctx->budget)
    return tm_fail(ctx, TM_E_BUDGET, "allocation exceeds the HBM budget");
  cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
  if (e != cudaSuccess) return tm_cuda_check(ctx, e, "cudaMallocAsync");
  ctx->in_use += bytes;
  return TM_OK;
}

void tm_free(tm_ctx* ctx, void* p, size_t bytes) {
  if (!p) return;
  if (bytes == 0) bytes = 16;
  cudaFreeAsync(p, ctx->stream);
  ctx->in_use -= std::min(ctx->in_use, bytes);
}

static const char* status_where(int w) {
  switch (w) {
    case 1: return "positions";
    case 2: return "cell grid";
    case 3: return "pair terms (sums out of range)";
    case 100: case 101: case 102: return "tensor-core GEMM";
    default: return "kernel";
  }
}

int tm_sync_status(tm_ctx* ctx, const char* what) {
  int rc = tm_cuda_check(ctx, cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(tm_dev_status),
                                              cudaMemcpyDeviceToHost, ctx->stream),
                         what);
  if (rc) return rc;
  if ((rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), what))) return rc;
  const tm_dev_status s = *ctx->h_status;
  if (s.code) {
    cudaMemsetAsync(ctx->d_status, 0, sizeof(tm_dev_status), ctx->stream);
    return tm_fail(ctx, s.code, std::string(what) + ": device status " + std::to_string(s.code) +
                                    " in " + status_where(s.where) + " (detail " +
                                    std::to_string(s.detail) + ")");
  }
  return TM_OK;
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
extern "C" int tm_ctx_create(int device, size_t budget, tm_ctx** out) {
  *out = nullptr;
  tm_ctx* c = new tm_ctx();
  c->device = device;
  c->budget = budget;
  int rc;
  if ((rc = tm_cuda_check(c, cudaSetDevice(device), "cudaSetDevice")) ||
      (rc = tm_cuda_check(c, cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount,
                                                    device), "SM count"))) {
    delete c;
    return rc;
  }
  if ((rc = tm_cuda_check(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream"))) {
    delete c;
    return rc;
  }
  c->own_stream = true;
  if ((rc = tm_cuda_check(c, cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking), "aux stream")) ||
      (rc = tm_cuda_check(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "event")) ||
      (rc = tm_cuda_check(c, cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "event"))) {
    delete c;
    return rc;
  }
  if ((rc = tm_cuda_check(c, cudaMalloc(&c->d_status, sizeof(tm_dev_status)), "status")) ||
      (rc = tm_cuda_check(c, cudaMallocHost(&c->h_status, sizeof(tm_dev_status)), "status")) ||
      (rc = tm_cuda_check(c, cudaMemset(c->d_status, 0, sizeof(tm_dev_status)), "status"))) {
    delete c;
    return rc;
  }
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
          cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    c->encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  *out = c;
  return TM_OK;
}

extern "C" int tm_ctx_destroy(tm_ctx* c) {
  if (!c) return TM_OK;
  cudaStreamSynchronize(c->stream);
  cudaStreamSynchronize(c->aux);
  cudaFree(c->d_status);
  cudaFreeHost(c->h_status);
  if (c->own_stream) cudaStreamDestroy(c->stream);
  cudaStreamDestroy(c->aux);
  cudaEventDestroy(c->ev_fork);
  cudaEventDestroy(c->ev_join);
  delete c;
  return TM_OK;
}

extern "C" int tm_ctx_set_stream(tm_ctx* c, void* s) {
  if (!c) return TM_E_ARG;
  cudaStreamSynchronize(c->stream);
  if (s) {
    if (c->own_stream) cudaStreamDestroy(c->stream);
    c->stream = (cudaStream_t)s;
    c->own_stream = false;
  }
  return TM_OK;
}

extern "C" void* tm_ctx_stream(tm_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" int tm_ctx_last_error(tm_ctx* c, char* buf, int len) {
  if (!c || !buf || len <= 0) return TM_E_ARG;
  snprintf(buf, (size_t)len, "%s", c->err.c_str());
  return TM_OK;
}

extern "C" size_t tm_ctx_bytes_in_use(tm_ctx* c) { return c ? c->in_use : 0; }
extern "C" int64_t tm_ctx_launch_count(tm_ctx* c) { return c ? c->launches : 0; }

// ---------------------------------------------------------------------------
// model
// ---------------------------------------------------------------------------
// Polynomial for erfcx(x) = exp(x^2) erfc(x) on [xa, xb] (the pair kernel forms
// erfc(x) = exp(-x^2) P(t) and reuses exp(-x^2) in the force term): Chebyshev
// interpolation at n + 1 nodes (erfcx is smooth, the coefficients fall off
// fast), converted to monomials in t = (2x - xa - xb) / (xb - xa) for Horner's
// rule. The smallest n <= 10 whose double-precision evaluation on 2001 points
// of the range is within 5e-8 relative is kept (FP32 evaluation adds about one
// ulp, 6e-8). A range that needs more keeps erfcf.
static void fit_erfcx(double xa, double xb, tm_consts& k) {
  k.erfc_n = 0;
  for (int q = 0; q < 11; ++q) k.erfc_c[q] = 0.f;
  if (!(xb > xa) || xa < 0.0 || xb > 9.0) return;
  auto erfcx = [](double x) { return exp(x * x) * erfc(x); };
  for (int n = 4; n <= 10; ++n) {
    double cheb[13] = {0}, mono[13] = {0};
    for (int j = 0; j <= n; ++j) {
      const double th = M_PI * (j + 0.5) / (n + 1);
      const double f = erfcx(0.5 * (xb - xa) * cos(th) + 0.5 * (xa + xb));
      for (int c = 0; c <= n; ++c) cheb[c] += 2.0 / (n + 1) * f * cos(c * th);
    }
    cheb[0] *= 0.5;
    // T_c as monomials: T_0 = 1, T_1 = t, T_{c+1} = 2 t T_c - T_{c-1}
    double Tm1[13] = {0}, T0[13] = {0}, T1[13] = {0};
    T0[0] = 1.0;
    for (int c = 0; c <= n; ++c) {
      for (int e = 0; e <= n; ++e) mono[e] += cheb[c] * T0[e];
      const double two = c == 0 ? 1.0 : 2.0;
      for (int e = 0; e <= 12; ++e) T1[e] = (e > 0 ? two * T0[e - 1] : 0.0) - Tm1[e];
      for (int e = 0; e <= 12; ++e) { Tm1[e] = T0[e]; T0[e] = T1[e]; }
    }
    double worst = 0.0;
    for (int q = 0; q <= 2000; ++q) {
      const double x = xa + (xb - xa) * q / 2000.0, t = (2.0 * x - xa - xb) / (xb - xa);
      double p = 0.0;
      for (int e = n; e >= 0; --e) p = p * t + mono[e];
      worst = fmax(worst, fabs(p / erfcx(x) - 1.0));
    }
    if (worst < 5e-8) {
      for (int e = 0; e <= n; ++e) k.erfc_c[e] = (float)mono[e];
      k.erfc_s = (float)(2.0 / (xb - xa));
      k.erfc_o = (float)(-(xa + xb) / (xb - xa));
      k.erfc_n = n;
      return;
    }
  }
}

static double dsf_val(double r, double rc, double alpha) {
  if (r > rc) return 0.0;
  const double xx = alpha * rc, zz = erfc(xx) / rc, yy = 1.1283791671 * alpha * exp(-xx * xx) / rc;
  return erfc(alpha * r) / r - zz + (r - rc) * (zz / rc + yy);
}
static double dsf_grad(double r, double rc, double alpha) {
  if (r > rc) return 0.0;
  const double xx = alpha * rc, zz = erfc(xx) / rc, yy = 1.1283791671 * alpha * exp(-xx * xx) / rc;
  return -((erfc(alpha * r) / r / r + 1.1283791671 * alpha * exp(-alpha * r * alpha * r) / r) -
           (zz / rc + yy));
}

static const double kBohr = 1.889725989;           // PhysicalData.py:30
static const double kJph = 2625.499638 * 1000.0;   // PhysicalData.py:36-37
static const double kC6[11] = {0, 0.14, 0.08, 1.16, 1.61, 3.13, 1.75, 1.23, 0.70, 0.75, 0.63};
static const double kR0[11] = {0, 1.001, 1.012, 0.825, 1.408, 1.485, 1.452, 1.397, 1.342, 1.287, 1.243};

extern "C" int tm_model_create(tm_ctx* ctx, const tm_model_desc* d, tm_model** out) {
  *out = nullptr;
  if (!ctx || !d) return TM_E_ARG;
  if (d->n_elements < 1 || d->n_elements > TM_MAX_ELE)
    return tm_fail(ctx, TM_E_ARG, "n_elements must be 1..8");
  for (int e = 0; e < d->n_elements; ++e) {
    if (d->elements[e] < 1 || d->elements[e] > 10)
      return tm_fail(ctx, TM_E_UNSUPPORTED, "elements must be Z = 1..10 (vdW tables)");
    if (e && d->elements[e] <= d->elements[e - 1])
      return tm_fail(ctx, TM_E_ARG, "elements must be sorted and unique");
  }
  if (d->n_hidden < 1 || d->n_hidden > 3)
    return tm_fail(ctx, TM_E_UNSUPPORTED, "1 to 3 hidden layers are supported");
  if (d->n_r_rs < 1 || d->n_r_rs > 32 || d->n_a_rs != 8 || d->n_a_as != 8)
    return tm_fail(ctx, TM_E_UNSUPPORTED, "AN1_num_r_Rs <= 32, AN1_num_a_Rs = AN1_num_a_As = 8");
  if (d->ee_cut_on != 0.0)
    return tm_fail(ctx, TM_E_ARG, "EECutoffOn should equal to zero in DSF_elu");
  if (!(d->a_rc > 0 && d->a_rc <= d->r_rc)) return tm_fail(ctx, TM_E_ARG, "need 0 < AN1_a_Rc <= AN1_r_Rc");
  if (d->precision != TM_PREC_FP32 && d->precision != TM_PREC_BF16)
    return tm_fail(ctx, TM_E_ARG, "precision");
  tm_model* m = new tm_model();
  m->ctx = ctx;
  m->desc = *d;
  tm_consts& k = m->k;
  memset(&k, 0, sizeof(k));
  k.nele = d->n_elements;
  k.nelep = k.nele * (k.nele + 1) / 2;
  k.nr = d->n_r_rs;
  k.na_rs = 8;
  k.na_as = 8;
  k.D = k.nele * k.nr + k.nelep * 64;
  k.Dp = ((k.D + TM_BN - 1) / TM_BN) * TM_BN;
  k.act = d->activation;
  k.alpha_sig = (float)d->sigmoid_alpha;
  k.r_rc = (float)d->r_rc;
  k.a_rc = (float)d->a_rc;
  k.eta = (float)d->eta;
  k.zeta = (float)d->zeta;
  k.zeta_pow2 = d->zeta == 8.0 ? 1 : 0;
  k.pi_tf = 3.14159265359f;   // RawSymFunc.py:935-936, 1799
  for (int n = 0; n < k.nr; ++n) k.rs_r[n] = (float)(d->r_rc * n / k.nr);
  for (int n = 0; n < 8; ++n) {
    k.rs_a[n] = (float)(d->a_rc * n / 8.0);
    const double th = 2.0 * M_PI * n / 8.0;
    k.cos_th[n] = (float)cos(th);
    k.sin_th[n] = (float)sin(th);
  }
  k.two_1mz = (float)pow(2.0, 1.0 - d->zeta);
  auto lo_of = [](double v) { return (float)(v - (double)(float)v); };
  for (int n = 0; n < k.nr; ++n) k.rs_r_lo[n] = lo_of(d->r_rc * n / k.nr);
  for (int n = 0; n < 8; ++n) {
    const double th = 2.0 * M_PI * n / 8.0;
    k.rs_a_lo[n] = lo_of(d->a_rc * n / 8.0);
    k.cos_th_lo[n] = lo_of(cos(th));
    k.sin_th_lo[n] = lo_of(sin(th));
  }
  k.r_rc_hi = (float)d->r_rc;
  k.r_rc_lo = lo_of(d->r_rc);
  k.a_rc_hi = (float)d->a_rc;
  k.a_rc_lo = lo_of(d->a_rc);
  // 0.5 (cos(pi_tf r / Rc) + 1) = sin^2(pi_tf (Rc - r) / (2 Rc) + (pi - pi_tf) / 2);
  // |pi - pi_tf| / 2 < 1.1e-13 is dropped
  const double cr = 3.14159265359 / (2.0 * d->r_rc), ca = 3.14159265359 / (2.0 * d->a_rc);
  k.cr_hi = (float)cr;
  k.cr_lo = lo_of(cr);
  k.ca_hi = (float)ca;
  k.ca_lo = lo_of(ca);
  int p = 0;
  for (int a = 0; a < k.nele; ++a)
    for (int b = a; b < k.nele; ++b) {
      k.elepair[a][b] = p;
      k.elepair[b][a] = p;
      ++p;
    }
  // TFBehlerParinelloSymEE.py:719-729, RawSymFunc.py:1323-1324
  const double alpha = d->dsf_alpha / kBohr, r_lr = d->ee_cut_off * kBohr, r_sr = d->elu_width * kBohr;
  fit_erfcx(alpha * r_sr * (1.0 - 1e-6), alpha * r_lr * (1.0 + 1e-6), k);
  k.bohr = (float)kBohr;
  k.alpha = (float)alpha;
  k.r_lr = (float)r_lr;
  k.r_sr = (float)r_sr;
  k.elu_shift = (float)dsf_val(r_sr, r_lr, alpha);
  k.elu_a = (float)dsf_grad(r_sr, r_lr, alpha);
  k.zz = (float)(erfc(alpha * r_lr) / r_lr);
  k.yy = (float)(1.1283791671 * alpha * exp(-alpha * r_lr * alpha * r_lr) / r_lr);
  k.vdw_width = (float)(d->poly_width * kBohr);
  k.vdw_begin = (float)(d->ee_cut_on * kBohr);
  for (int e = 0; e < k.nele; ++e) {
    const int z = d->elements[e];
    k.c6[e] = (float)(kC6[z] * pow(kBohr * 10.0, 6.0) / kJph);
    k.r0[e] = (float)(kR0[z] * kBohr);
  }
  k.r_rc_d = d->r_rc;
  k.a_rc_d = d->a_rc;
  k.ree_d = d->ee_cut_off;
  k.ree = (float)d->ee_cut_off;
  k.add_ecc = d->add_ecc ? 1 : 0;
  k.has_vdw = d->has_vdw ? 1 : 0;
  m->nlayer = d->n_hidden;
  int hmax = 0;
  for (int l = 0; l < d->n_hidden; ++l) {
    if (d->hidden[l] < 1) { delete m; return tm_fail(ctx, TM_E_ARG, "hidden width"); }
    hmax = std::max(hmax, d->hidden[l]);
  }
  m->H = ((hmax + TM_BN - 1) / TM_BN) * TM_BN;
  m->elem_size = d->precision == TM_PREC_FP32 ? 4 : 2;
  m->layers.resize((size_t)2 * k.nele * (m->nlayer + 1));
  *out = m;
  return TM_OK;
}

extern "C" int tm_model_descriptor_width(const tm_model* m) { return m ? m->k.D : -1; }

extern "C" int tm_model_erfc_poly(const tm_model* m, float* coeffs, int* n, float* scale,
                                  float* offset, double* x0, double* x1) {
  if (!m || !coeffs || !n || !scale || !offset || !x0 || !x1) return TM_E_ARG;
  for (int e = 0; e < 11; ++e) coeffs[e] = m->k.erfc_c[e];
  *n = m->k.erfc_n;
  *scale = m->k.erfc_s;
  *offset = m->k.erfc_o;
  const double alpha = m->desc.dsf_alpha / kBohr;
  *x0 = alpha * m->desc.elu_width * kBohr;
  *x1 = alpha * m->desc.ee_cut_off * kBohr;
  return TM_OK;
}

extern "C" int tm_model_set_layer(tm_model* m, int net, int e, int layer, const double* W,
                                  const double* b, int fan_in, int fan_out) {
  if (!m || !W || !b || net < 0 || net > 1 || e < 0 || e >= m->k.nele || layer < 0 ||
      layer > m->nlayer)
    return tm_fail(m ? m->ctx : nullptr, TM_E_ARG, "set_layer index");
  const int want_in = layer == 0 ? m->k.D : m->desc.hidden[layer - 1];
  const int want_out = layer == m->nlayer ? 1 : m->desc.hidden[layer];
  if (fan_in != want_in || fan_out != want_out)
    return tm_fail(m->ctx, TM_E_ARG, "layer shape does not match the model description");
  tm_layer_host& L = m->layers[((size_t)net * m->k.nele + e) * (m->nlayer + 1) + layer];
  L.W.assign(W, W + (size_t)fan_in * fan_out);
  L.b.assign(b, b + fan_out);
  L.fan_in = fan_in;
  L.fan_out = fan_out;
  L.set = true;
  m->final_ = false;
  return TM_OK;
}

// pack one matrix into hi/lo (tf32) or bf16 device layout
static int upload_split(tm_model* m, const std::vector<float>& host, void* out[2]) {
  tm_ctx* ctx = m->ctx;
  const size_t n = host.size();
  int rc;
  if (m->desc.precision == TM_PREC_FP32) {
    std::vector<float> hi(n), lo(n);
    for (size_t q = 0; q < n; ++q) tm_tf32_split(host[q], hi[q], lo[q]);
    if ((rc = tm_alloc(ctx, &out[0], n * 4)) || (rc = tm_alloc(ctx, &out[1], n * 4))) return rc;
    cudaMemcpyAsync(out[0], hi.data(), n * 4, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(out[1], lo.data(), n * 4, cudaMemcpyHostToDevice, ctx->stream);
    return tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "upload");
  }
  std::vector<__nv_bfloat16> b(n);
  for (size_t q = 0; q < n; ++q) b[q] = __float2bfloat16_rn(host[q]);
  if ((rc = tm_alloc(ctx, &out[0], n * 2))) return rc;
  out[1] = out[0];
  cudaMemcpyAsync(out[0], b.data(), n * 2, cudaMemcpyHostToDevice, ctx->stream);
  return tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "upload");
}

extern "C" int tm_model_finalize(tm_model* m) {
  if (!m) return TM_E_ARG;
  tm_ctx* ctx = m->ctx;
  for (auto& L : m->layers)
    if (!L.set) return tm_fail(ctx, TM_E_STATE, "every layer of both networks must be set");
  const int nele = m->k.nele, L = m->nlayer, H = m->H, Dp = m->k.Dp;
  auto layer = [&](int net, int e, int l) -> tm_layer_host& {
    return m->layers[((size_t)net * nele + e) * (L + 1) + l];
  };
  int rc;
  // relu kinks: FP32 mode recomputes near-kink units in FP64 (tm_gemm.cu)
  m->kink = m->desc.precision == TM_PREC_FP32 && m->desc.activation == TM_ACT_RELU;
  for (int l = 0; l < L; ++l) {
    const int Kin = l == 0 ? Dp : H;
    std::vector<float> fwd((size_t)2 * nele * H * Kin, 0.f), bwd((size_t)2 * nele * Kin * H, 0.f);
    std::vector<float> bias((size_t)2 * nele * H, 0.f);
    for (int net = 0; net < 2; ++net)
      for (int e = 0; e < nele; ++e) {
        const tm_layer_host& Lh = layer(net, e, l);
        const size_t blk = (size_t)net * nele + e;
        for (int i = 0; i < Lh.fan_in; ++i)
          for (int o = 0; o < Lh.fan_out; ++o) {
            const float w = (float)Lh.W[(size_t)i * Lh.fan_out + o];
            fwd[(blk * H + o) * Kin + i] = w;     // W^T: [Nout][Kin]
            bwd[(blk * Kin + i) * H + o] = w;     // W:   [Kin][Nout]
          }
        for (int o = 0; o < Lh.fan_out; ++o) bias[blk * H + o] = (float)Lh.b[o];
      }
    if ((rc = upload_split(m, fwd, m->w_fwd[l])) || (rc = upload_split(m, bwd, m->w_bwd[l]))) return rc;
    if (m->kink && l == L - 1) {
      // the output weights folded into the last layer's backward weights
      // (products in FP64, then split)
      std::vector<float> bwdf(bwd.size(), 0.f);
      for (int net = 0; net < 2; ++net)
        for (int e = 0; e < nele; ++e) {
          const tm_layer_host& Lh = layer(net, e, l);
          const tm_layer_host& Lo = layer(net, e, L);
          const size_t blk = (size_t)net * nele + e;
          for (int i = 0; i < Lh.fan_in; ++i)
            for (int o = 0; o < Lh.fan_out; ++o)
              bwdf[(blk * Kin + i) * H + o] = (float)(Lh.W[(size_t)i * Lh.fan_out + o] * Lo.W[o]);
        }
      if (m->w_bwd_fold[0]) {   // finalized before: replace
        tm_free(ctx, m->w_bwd_fold[0], bwdf.size() * 4);
        tm_free(ctx, m->w_bwd_fold[1], bwdf.size() * 4);
      }
      if ((rc = upload_split(m, bwdf, m->w_bwd_fold))) return rc;
    }
    if (m->kink) {
      // the weights and biases as given (FP64) and the norm of each unit's
      // weight vector, for the relu refinement (tm_gemm.cu)
      std::vector<float2> w2((size_t)2 * nele * H * Kin, make_float2(0.f, 0.f)),
          b2((size_t)2 * nele * H, make_float2(0.f, 0.f));
      auto pair = [](double v) {
        const float h = (float)v;
        return make_float2(h, (float)(v - (double)h));
      };
      std::vector<float> wn((size_t)2 * nele * H, 0.f);
      for (int net = 0; net < 2; ++net)
        for (int e = 0; e < nele; ++e) {
          const tm_layer_host& Lh = layer(net, e, l);
          const size_t blk = (size_t)net * nele + e;
          for (int o = 0; o < Lh.fan_out; ++o) {
            double ss = 0.0;
            for (int i = 0; i < Lh.fan_in; ++i) {
              const double w = Lh.W[(size_t)i * Lh.fan_out + o];
              w2[(blk * H + o) * Kin + i] = pair(w);
              ss += w * w;
            }
            wn[blk * H + o] = (float)sqrt(ss);
            b2[blk * H + o] = pair(Lh.b[o]);
          }
        }
      if (m->kw2[l]) {   // finalized before: replace
        tm_free(ctx, m->kw2[l], w2.size() * 8);
        tm_free(ctx, m->kb2[l], b2.size() * 8);
        tm_free(ctx, m->kwn[l], wn.size() * 4);
      }
      if ((rc = tm_alloc(ctx, (void**)&m->kw2[l], w2.size() * 8)) ||
          (rc = tm_alloc(ctx, (void**)&m->kb2[l], b2.size() * 8)) ||
          (rc = tm_alloc(ctx, (void**)&m->kwn[l], wn.size() * 4)))
        return rc;
      cudaMemcpyAsync(m->kw2[l], w2.data(), w2.size() * 8, cudaMemcpyHostToDevice, ctx->stream);
      cudaMemcpyAsync(m->kb2[l], b2.data(), b2.size() * 8, cudaMemcpyHostToDevice, ctx->stream);
      cudaMemcpyAsync(m->kwn[l], wn.data(), wn.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
      if ((rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "finalize"))) return rc;
    }
    if ((rc = tm_alloc(ctx, (void**)&m->bias[l], bias.size() * 4))) return rc;
    cudaMemcpyAsync(m->bias[l], bias.data(), bias.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    const int eb = (int)m->elem_size;
    const uint32_t bn = (uint32_t)tm_gemm_bn(m->desc.precision);   // B tile rows
    if ((rc = tm_make_tmap(ctx, &m->tm_wf[l][0], m->w_fwd[l][0], eb, (uint64_t)2 * nele * H, Kin, bn)) ||
        (rc = tm_make_tmap(ctx, &m->tm_wf[l][1], m->w_fwd[l][1], eb, (uint64_t)2 * nele * H, Kin, bn)) ||
        (rc = tm_make_tmap(ctx, &m->tm_wb[l][0], m->w_bwd[l][0], eb, (uint64_t)2 * nele * Kin, H, bn)) ||
        (rc = tm_make_tmap(ctx, &m->tm_wb[l][1], m->w_bwd[l][1], eb, (uint64_t)2 * nele * Kin, H, bn)))
      return rc;
    if (m->w_bwd_fold[0] && l == L - 1 &&
        ((rc = tm_make_tmap(ctx, &m->tm_wbf[0], m->w_bwd_fold[0], eb, (uint64_t)2 * nele * Kin, H, bn)) ||
         (rc = tm_make_tmap(ctx, &m->tm_wbf[1], m->w_bwd_fold[1], eb, (uint64_t)2 * nele * Kin, H, bn))))
      return rc;
  }
  std::vector<float> wout((size_t)2 * nele * H, 0.f);
  std::vector<double> bout((size_t)2 * nele, 0.0);
  for (int net = 0; net < 2; ++net)
    for (int e = 0; e < nele; ++e) {
      const tm_layer_host& Lh = layer(net, e, L);
      const size_t blk = (size_t)net * nele + e;
      for (int i = 0; i < Lh.fan_in; ++i) wout[blk * H + i] = (float)Lh.W[i];
      bout[blk] = Lh.b[0];
    }
  if ((rc = tm_alloc(ctx, (void**)&m->wout, wout.size() * 4)) ||
      (rc = tm_alloc(ctx, (void**)&m->bout, bout.size() * 8)))
    return rc;
  cudaMemcpyAsync(m->wout, wout.data(), wout.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
  cudaMemcpyAsync(m->bout, bout.data(), bout.size() * 8, cudaMemcpyHostToDevice, ctx->stream);
  if ((rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "finalize"))) return rc;
  m->final_ = true;
  return TM_OK;
}

extern "C" int tm_model_destroy(tm_model* m) {
  if (!m) return TM_OK;
  tm_ctx* ctx = m->ctx;
  const int nele = m->k.nele, H = m->H, Dp = m->k.Dp;
  for (int l = 0; l < m->nlayer; ++l) {
    const int Kin = l == 0 ? Dp : H;
    const size_t n = (size_t)2 * nele * H * Kin * m->elem_size;
    for (int s = 0; s < 2; ++s) {
      if (m->desc.precision == TM_PREC_BF16 && s == 1) continue;
      tm_free(ctx, m->w_fwd[l][s], n);
      tm_free(ctx, m->w_bwd[l][s], n);
    }
    tm_free(ctx, m->bias[l], (size_t)2 * nele * H * 4);
    if (m->kw2[l]) {
      tm_free(ctx, m->kw2[l], (size_t)2 * nele * H * Kin * 8);
      tm_free(ctx, m->kb2[l], (size_t)2 * nele * H * 8);
      tm_free(ctx, m->kwn[l], (size_t)2 * nele * H * 4);
    }
  }
  if (m->w_bwd_fold[0]) {
    const size_t nf = (size_t)2 * nele * (m->nlayer == 1 ? Dp : H) * H * 4;
    tm_free(ctx, m->w_bwd_fold[0], nf);
    tm_free(ctx, m->w_bwd_fold[1], nf);
  }
  tm_free(ctx, m->wout, (size_t)2 * nele * H * 4);
  tm_free(ctx, m->bout, (size_t)2 * nele * 8);
  cudaStreamSynchronize(ctx->stream);
  delete m;
  return TM_OK;
}

// ---------------------------------------------------------------------------
// system
// ---------------------------------------------------------------------------
struct AllocList {
  tm_system* s;
  int rc = 0;
  template <typename T>
  void get(T** p, size_t bytes) {
    if (rc) return;
    rc = tm_alloc(s->ctx, (void**)p, bytes);
    if (!rc) s->bytes += bytes;
  }
};

static void system_free(tm_system* s);

// Host-side tables of one layout: a batch of molecules in CSR order.
struct SysLayout {
  int N = 0, nmol = 0, Mpad = 0, ntiles = 0, nchunk = 0, ncell_cap = 0, ecell_cap = 0;
  std::vector<int32_t> Z, elem, row_of_atom, atom_of_row, tile_elem, mol, off32, mol_chunk;
  std::vector<int64_t> off;
  std::vector<int2> chunks;
};

static int build_layout(tm_system* s, int N, int nmol, const int32_t* Z, const int64_t* off,
                        SysLayout& L) {
  tm_ctx* ctx = s->ctx;
  const tm_consts& k = s->model->k;
  if (N <= 0 || nmol <= 0 || !Z || !off) return tm_fail(ctx, TM_E_ARG, "system args");
  if (off[0] != 0 || off[nmol] != N) return tm_fail(ctx, TM_E_ARG, "mol_offsets must span 0..natoms");
  for (int q = 0; q < nmol; ++q)
    if (off[q + 1] <= off[q]) return tm_fail(ctx, TM_E_ARG, "empty or unsorted molecule");
  if (N >= (1 << 27)) return tm_fail(ctx, TM_E_ARG, "too many atoms");
  L.N = N;
  L.nmol = nmol;
  L.Z.assign(Z, Z + N);
  L.off.assign(off, off + nmol + 1);
  // elements and element-sorted rows (each element padded to TM_BM rows)
  L.elem.resize(N);
  std::vector<int> count(k.nele, 0);
  for (int i = 0; i < N; ++i) {
    int e = -1;
    for (int q = 0; q < k.nele; ++q)
      if (s->model->desc.elements[q] == Z[i]) e = q;
    if (e < 0) return tm_fail(ctx, TM_E_ARG, "atom element not in the model");
    L.elem[i] = e;
    count[e]++;
  }
  std::vector<int> row_off(k.nele + 1, 0);
  for (int e = 0; e < k.nele; ++e) row_off[e + 1] = row_off[e] + ((count[e] + TM_BM - 1) / TM_BM) * TM_BM;
  L.Mpad = row_off[k.nele];
  L.ntiles = L.Mpad / TM_BM;
  L.row_of_atom.resize(N);
  L.atom_of_row.assign(L.Mpad, -1);
  std::vector<int> fill(k.nele, 0);
  for (int i = 0; i < N; ++i) {
    const int e = L.elem[i];
    const int r = row_off[e] + fill[e]++;
    L.row_of_atom[i] = r;
    L.atom_of_row[r] = i;
  }
  L.tile_elem.resize(L.ntiles);
  for (int e = 0; e < k.nele; ++e)
    for (int r = row_off[e]; r < row_off[e + 1]; r += TM_BM) L.tile_elem[r / TM_BM] = e;
  L.mol.resize(N);
  for (int q = 0; q < nmol; ++q)
    for (int64_t i = off[q]; i < off[q + 1]; ++i) L.mol[i] = q;
  L.off32.resize(nmol + 1);
  for (int q = 0; q <= nmol; ++q) L.off32[q] = (int32_t)off[q];
  // chunks of at most TM_CHUNK atoms of one molecule (two-level reductions)
  L.mol_chunk.assign(nmol + 1, 0);
  for (int q = 0; q < nmol; ++q) {
    L.mol_chunk[q] = (int32_t)L.chunks.size();
    for (int64_t b = off[q]; b < off[q + 1]; b += TM_CHUNK)
      L.chunks.push_back(make_int2((int)b, (int)std::min<int64_t>(b + TM_CHUNK, off[q + 1])));
  }
  L.mol_chunk[nmol] = (int32_t)L.chunks.size();
  L.nchunk = (int)L.chunks.size();
  // cell bounds: neighbour grid (open: at most 2n + 64 cells per molecule) and
  // Coulomb grid (about 24 atoms per cell; open: at most n/8 + 8 per molecule,
  // the device grows the cell size until a molecule fits within the bound)
  if (s->periodic) {
    long nc = 1, ne = 1;
    for (int d = 0; d < 3; ++d) {
      nc *= (long)floor(s->hpl[d] / k.r_rc_d);
      ne *= s->ee_dims[d];
    }
    L.ncell_cap = (int)nc;
    L.ecell_cap = (int)ne;
  } else {
    L.ncell_cap = 2 * N + 64 * nmol;
    L.ecell_cap = 0;
    for (int q = 0; q < nmol; ++q) L.ecell_cap += (int)((off[q + 1] - off[q]) / 8) + 8;
  }
  return TM_OK;
}

// Zero the descriptor rows of the padding rows (atom_of_row < 0), so that
// rows left from an earlier layout never reach the networks.
__global__ void k_zero_pad_rows(const int32_t* __restrict__ atom_of_row, int Mpad, int Dp,
                                float* __restrict__ g0, float* __restrict__ g1, int words,
                                float* __restrict__ gnorm2) {
  const int r = blockIdx.x;
  if (r >= Mpad || atom_of_row[r] >= 0) return;
  if (gnorm2 && threadIdx.x == 0) gnorm2[r] = 0.f;
  for (int c = threadIdx.x; c < words; c += blockDim.x) {
    g0[(size_t)r * words + c] = 0.f;
    if (g1) g1[(size_t)r * words + c] = 0.f;
  }
}

static int upload_layout(tm_system* s, SysLayout& L) {
  tm_ctx* ctx = s->ctx;
  const tm_model* m = s->model;
  if (L.N > s->N_cap || L.nmol > s->nmol_cap || L.Mpad > s->Mpad_cap || L.nchunk > s->nchunk_cap ||
      L.ncell_cap > s->ncell_alloc || L.ecell_cap > s->ecell_alloc)
    return tm_fail(ctx, TM_E_CAPACITY, "layout exceeds the system's capacity");
  s->N = L.N;
  s->nmol = L.nmol;
  s->Z = L.Z;
  s->off = L.off;
  s->elem_h = L.elem;
  s->Mpad = L.Mpad;
  s->ntiles = L.ntiles;
  s->row_of_atom_h = L.row_of_atom;
  s->tile_elem_h = L.tile_elem;
  s->nchunk = L.nchunk;
  s->ncell_cap = L.ncell_cap;
  s->ecell_cap = L.ecell_cap;
  s->nlist_valid = false;
  cudaStream_t st = ctx->stream;
  const int N = L.N, nmol = L.nmol;
  // The tables go through one pinned staging buffer of the system (no
  // pageable-copy staging, no stream sync); before it is refilled, the copies
  // of the previous upload are waited for (normally long done).
  struct Part { void* dst; const void* src; size_t bytes; };
  const Part parts[] = {
      {s->row_of_atom, L.row_of_atom.data(), sizeof(int32_t) * N},
      {s->atom_of_row, L.atom_of_row.data(), sizeof(int32_t) * L.Mpad},
      {s->tile_elem, L.tile_elem.data(), sizeof(int32_t) * L.ntiles},
      {s->d_Z, L.Z.data(), sizeof(int32_t) * N},
      {s->d_elem, L.elem.data(), sizeof(int32_t) * N},
      {s->d_mol, L.mol.data(), sizeof(int32_t) * N},
      {s->d_off, L.off32.data(), sizeof(int32_t) * (nmol + 1)},
      {s->d_chunk, L.chunks.data(), sizeof(int2) * L.nchunk},
      {s->d_mol_chunk, L.mol_chunk.data(), sizeof(int32_t) * (nmol + 1)}};
  size_t total = 0;
  for (const Part& p : parts) total += (p.bytes + 15) & ~(size_t)15;
  int rc;
  if (s->stage_ev && (rc = tm_cuda_check(ctx, cudaEventSynchronize(s->stage_ev), "upload staging")))
    return rc;
  if (total > s->h_stage_bytes) {
    if (s->h_stage) cudaFreeHost(s->h_stage);
    s->h_stage = nullptr;
    s->h_stage_bytes = 0;
    if ((rc = tm_cuda_check(ctx, cudaMallocHost(&s->h_stage, total), "upload staging"))) return rc;
    s->h_stage_bytes = total;
  }
  if (!s->stage_ev &&
      (rc = tm_cuda_check(ctx, cudaEventCreateWithFlags(&s->stage_ev, cudaEventDisableTiming), "event")))
    return rc;
  size_t o = 0;
  for (const Part& p : parts) {
    uint8_t* h = static_cast<uint8_t*>(s->h_stage) + o;
    memcpy(h, p.src, p.bytes);
    if (p.bytes) cudaMemcpyAsync(p.dst, h, p.bytes, cudaMemcpyHostToDevice, st);
    o += (p.bytes + 15) & ~(size_t)15;
  }
  cudaEventRecord(s->stage_ev, st);
  const bool split = m->desc.precision == TM_PREC_FP32;
  const int words = (int)(m->k.Dp * m->elem_size / 4);
  k_zero_pad_rows<<<L.Mpad, 128, 0, st>>>(s->atom_of_row, L.Mpad, m->k.Dp, (float*)s->G[0],
                                          split ? (float*)s->G[1] : nullptr, words, s->kink_g2);
  ctx->launches++;
  return tm_cuda_check(ctx, cudaGetLastError(), "system upload");
}

// Device buffers for up to N_cap atoms / nmol_cap molecules and the given
// cell, chunk and row bounds; any layout within them can be uploaded later.
static int system_alloc(tm_system* s, int N_cap, int nmol_cap, int Mpad_cap, int nchunk_cap,
                        int ncell_alloc, int ecell_alloc) {
  tm_ctx* ctx = s->ctx;
  const tm_model* m = s->model;
  s->N_cap = N_cap;
  s->nmol_cap = nmol_cap;
  s->Mpad_cap = Mpad_cap;
  s->nchunk_cap = nchunk_cap;
  s->ncell_alloc = ncell_alloc;
  s->ecell_alloc = ecell_alloc;
  const int N = N_cap, nmol = nmol_cap;
  const int H = m->H, Dp = m->k.Dp;
  const size_t es = m->elem_size;
  const size_t Mp = Mpad_cap;
  AllocList A{s};
  A.get(&s->row_of_atom, sizeof(int32_t) * N);
  A.get(&s->atom_of_row, sizeof(int32_t) * Mp);
  A.get(&s->tile_elem, sizeof(int32_t) * (Mp / TM_BM));
  A.get(&s->d_Z, sizeof(int32_t) * N);
  A.get(&s->d_elem, sizeof(int32_t) * N);
  A.get(&s->d_mol, sizeof(int32_t) * N);
  A.get(&s->d_off, sizeof(int32_t) * (nmol + 1));
  A.get(&s->d_x, sizeof(double) * 3 * N);
  A.get(&s->d_xhi, sizeof(float4) * N);
  A.get(&s->d_xlo, sizeof(float4) * N);
  A.get(&s->d_x_at_build, sizeof(double) * 3 * N);
  A.get(&s->d_grid, sizeof(tm_grid) * nmol);
  A.get(&s->d_ncell, sizeof(int32_t));
  A.get(&s->d_ncell_m, sizeof(int32_t) * nmol);
  A.get(&s->d_need, sizeof(int32_t) * 2);
  A.get(&s->d_cell_cnt, sizeof(int32_t) * (ncell_alloc + 1));
  A.get(&s->d_cell_start, sizeof(int32_t) * (ncell_alloc + 1));
  A.get(&s->d_cell_atoms, sizeof(int32_t) * N);
  A.get(&s->d_cell_of_atom, sizeof(int32_t) * N);
  A.get(&s->d_sort_tmp, sizeof(int32_t) * N);
  A.get(&s->d_scan_tmp, sizeof(int32_t) * 4096);
  A.get(&s->d_sort_tmp2, sizeof(int32_t) * N);
  A.get(&s->d_scan_tmp2, sizeof(int32_t) * 4096);
  A.get(&s->d_ccnt, sizeof(int32_t) * N);
  A.get(&s->d_cand, sizeof(uint32_t) * (size_t)N * s->KC);
  A.get(&s->d_need_c, sizeof(int32_t) * 2);
  A.get(&s->d_disp, sizeof(unsigned long long));
  A.get(&s->d_chunk, sizeof(int2) * nchunk_cap);
  A.get(&s->d_mol_chunk, sizeof(int32_t) * (nmol + 1));
  A.get(&s->d_part, sizeof(double) * 8 * nchunk_cap);
  A.get(&s->d_cbox, sizeof(float) * 8 * nchunk_cap);
  A.get(&s->d_egrid, sizeof(tm_grid) * nmol);
  A.get(&s->d_encell, sizeof(int32_t));
  A.get(&s->d_encell_m, sizeof(int32_t) * nmol);
  A.get(&s->d_ecell_cnt, sizeof(int32_t) * (ecell_alloc + 1));
  A.get(&s->d_ecell_start, sizeof(int32_t) * (ecell_alloc + 1));
  A.get(&s->d_ecell_atoms, sizeof(int32_t) * N);
  A.get(&s->d_ecell_of_atom, sizeof(int32_t) * N);
  A.get(&s->d_epos, sizeof(int32_t) * N);
  A.get(&s->d_exhi, sizeof(float4) * N);
  A.get(&s->d_exlo, sizeof(float4) * N);
  A.get(&s->d_cacc, sizeof(unsigned long long) * 5 * (size_t)N);
  A.get(&s->d_eblk, sizeof(int4) * ((size_t)N / 32 + ecell_alloc + 1));
  A.get(&s->d_neblk, sizeof(int32_t));
  A.get(&s->d_cnt_r, sizeof(int32_t) * N);
  A.get(&s->d_cnt_a, sizeof(int32_t) * N);
  A.get(&s->d_nbr_r, sizeof(uint32_t) * (size_t)N * s->KR);
  A.get(&s->d_nbr_a, sizeof(uint32_t) * (size_t)N * s->KA);
  A.get(&s->d_rev_r, sizeof(int32_t) * (size_t)N * s->KR);
  A.get(&s->d_rev_a, sizeof(int32_t) * (size_t)N * s->KA);
  A.get(&s->d_sr, sizeof(float) * (size_t)N * s->KR);
  A.get(&s->d_va, sizeof(float4) * (size_t)N * s->KA);
  for (int h = 0; h < 2; ++h) {
    if (m->desc.precision == TM_PREC_BF16 && h == 1) {
      s->G[1] = s->G[0]; s->H1[1] = s->H1[0]; s->H2[1] = s->H2[0]; s->G3[1] = s->G3[0];
      continue;
    }
    A.get(&s->G[h], Mp * Dp * es);
    A.get(&s->H1[h], 2 * Mp * H * es);
    A.get(&s->H2[h], 2 * Mp * H * es);
    A.get(&s->G3[h], 2 * Mp * H * es);
  }
  A.get(&s->dEdG, sizeof(float) * 2 * Mp * Dp);
  if (m->k.act == TM_ACT_RELU) A.get(&s->relu_mask, sizeof(uint32_t) * TM_MAX_HIDDEN * 2 * Mp * (H / 32));
  A.get(&s->epart, sizeof(float) * 2 * Mp * tm_gemm_row_parts(m->desc.precision, H));
  if (m->kink) {
    const size_t parts = tm_gemm_row_parts(m->desc.precision, H);
    A.get(&s->kink_g2, sizeof(float) * Mp);
    A.get(&s->kink_h2[0], sizeof(float) * 2 * Mp * parts);
    A.get(&s->kink_h2[1], sizeof(float) * 2 * Mp * parts);
    A.get(&s->kink_mask, sizeof(uint32_t) * 2 * Mp * (H / 32));
    A.get(&s->kink_count, sizeof(unsigned long long));
    A.get(&s->kink_rows, sizeof(uint32_t) * 2 * Mp * parts);
    A.get(&s->kink_nrows, sizeof(uint32_t) * TM_KINK_LAYERS);
  }
  A.get(&s->d_Eatom, sizeof(double) * N);
  A.get(&s->d_qraw, sizeof(float) * N);
  A.get(&s->d_q, sizeof(float) * N);
  A.get(&s->d_dEdq, sizeof(float) * N);
  A.get(&s->d_fself, sizeof(float4) * N);
  A.get(&s->d_fcv, sizeof(float4) * N);
  A.get(&s->d_ecv, sizeof(double) * 2 * N);
  A.get(&s->d_F, sizeof(double) * 3 * N);
  A.get(&s->d_mol_E, sizeof(double) * 4 * nmol);
  A.get(&s->d_mol_aux, sizeof(double) * 8 * nmol);
  if (A.rc) return A.rc;
  cudaStream_t st = ctx->stream;
  for (int h = 0; h < 2; ++h) {
    if (m->desc.precision == TM_PREC_BF16 && h == 1) break;
    cudaMemsetAsync(s->G[h], 0, Mp * Dp * es, st);
  }
  cudaMemsetAsync(s->d_x, 0, sizeof(double) * 3 * N, st);
  if (s->kink_g2) cudaMemsetAsync(s->kink_g2, 0, sizeof(float) * Mp, st);
  if (s->kink_count) cudaMemsetAsync(s->kink_count, 0, sizeof(unsigned long long), st);
  int rc;
  if ((rc = tm_cuda_check(ctx, cudaStreamSynchronize(st), "system alloc"))) return rc;
  const int eb = (int)es;
  for (int h = 0; h < 2; ++h) {
    if ((rc = tm_make_tmap(ctx, &s->tm_G[h], s->G[h], eb, Mp, Dp, TM_BM)) ||
        (rc = tm_make_tmap(ctx, &s->tm_H1[h], s->H1[h], eb, 2 * Mp, H, TM_BM)) ||
        (rc = tm_make_tmap(ctx, &s->tm_H2[h], s->H2[h], eb, 2 * Mp, H, TM_BM)) ||
        (rc = tm_make_tmap(ctx, &s->tm_G3[h], s->G3[h], eb, 2 * Mp, H, TM_BM)))
      return rc;
    if ((rc = tm_make_tmap(ctx, &s->ts_H1[h], s->H1[h], eb, 2 * Mp, H, 32)) ||
        (rc = tm_make_tmap(ctx, &s->ts_H2[h], s->H2[h], eb, 2 * Mp, H, 32)) ||
        (rc = tm_make_tmap(ctx, &s->ts_G3[h], s->G3[h], eb, 2 * Mp, H, 32)))
      return rc;
  }
  if ((rc = tm_make_tmap(ctx, &s->ts_dEdG, s->dEdG, 4, 2 * Mp, Dp, 32))) return rc;
  return TM_OK;
}

extern "C" int tm_system_create(tm_model* m, int N, int nmol, const int32_t* Z,
                                const int64_t* off, const double* cell, tm_system** out) {
  *out = nullptr;
  if (!m || !Z || !off || N <= 0 || nmol <= 0) return tm_fail(m ? m->ctx : nullptr, TM_E_ARG, "system args");
  tm_ctx* ctx = m->ctx;
  if (!m->final_) return tm_fail(ctx, TM_E_STATE, "model weights are not finalized");
  tm_system* s = new tm_system();
  s->model = m;
  s->ctx = ctx;
  const tm_consts& k = m->k;
  if (cell) {
    for (int q = 0; q < 9; ++q) s->lat[q] = cell[q];
    if (nmol != 1) { delete s; return tm_fail(ctx, TM_E_ARG, "a periodic system is one molecule"); }
    // any three lattice vectors (Periodic.py:12-24): the cells of both grids
    // are slices between lattice planes, binned by each atom's distance from
    // the planes through the origin (its coordinate along the plane normals)
    const double* a0 = cell;
    const double* a1 = cell + 3;
    const double* a2 = cell + 6;
    auto cross = [](const double* u, const double* v, double* w) {
      w[0] = u[1] * v[2] - u[2] * v[1];
      w[1] = u[2] * v[0] - u[0] * v[2];
      w[2] = u[0] * v[1] - u[1] * v[0];
    };
    double c[3][3];
    cross(a1, a2, c[0]);
    cross(a2, a0, c[1]);
    cross(a0, a1, c[2]);
    const double vol = a0[0] * c[0][0] + a0[1] * c[0][1] + a0[2] * c[0][2];
    if (!(std::fabs(vol) > 0.0) || !std::isfinite(vol)) {
      delete s;
      return tm_fail(ctx, TM_E_ARG, "lattice vectors are linearly dependent");
    }
    s->ortho = cell[1] == 0 && cell[2] == 0 && cell[3] == 0 && cell[5] == 0 && cell[6] == 0 &&
               cell[7] == 0 && cell[0] > 0 && cell[4] > 0 && cell[8] > 0;
    for (int d = 0; d < 3; ++d) {
      const double cn = std::sqrt(c[d][0] * c[d][0] + c[d][1] * c[d][1] + c[d][2] * c[d][2]);
      const double sg = vol > 0 ? 1.0 : -1.0;
      for (int e = 0; e < 3; ++e) {
        s->nrm[3 * d + e] = s->ortho ? (e == d ? 1.0 : 0.0) : sg * c[d][e] / cn;
        s->binv[3 * e + d] = c[d][e] / vol;
      }
      s->hpl[d] = s->ortho ? cell[4 * d] : std::fabs(vol) / cn;
    }
    const double hmin = std::min(s->hpl[0], std::min(s->hpl[1], s->hpl[2]));
    const double rmax = std::max(k.r_rc_d, k.ree_d);
    if (hmin < 2.0 * rmax) {
      // a small cell: evaluated as the smallest supercell whose plane
      // spacings are at least twice the largest cutoff
      int rep[3];
      long K = 1;
      for (int d = 0; d < 3; ++d) {
        rep[d] = std::max(1, (int)std::ceil(2.0 * rmax / s->hpl[d] * (1.0 + 1e-12)));
        K *= rep[d];
      }
      if (K > 4096 || (long)N * K >= (1L << 26)) {
        delete s;
        return tm_fail(ctx, TM_E_ARG, "cell too small for its cutoffs (more than 4096 copies)");
      }
      std::vector<double> sup(9);
      for (int d = 0; d < 3; ++d)
        for (int e = 0; e < 3; ++e) sup[3 * d + e] = rep[d] * cell[3 * d + e];
      std::vector<int32_t> Zs((size_t)N * K);
      for (long c = 0; c < K; ++c)
        for (int a = 0; a < N; ++a) Zs[c * N + a] = Z[a];
      const int64_t offs[2] = {0, (int64_t)N * K};
      delete s;
      tm_system* sup_s = nullptr;
      int rc = tm_system_create(m, (int)(N * K), 1, Zs.data(), offs, sup.data(), &sup_s);
      if (rc) return rc;
      for (int d = 0; d < 3; ++d) sup_s->rep[d] = rep[d];
      sup_s->K = (int)K;
      sup_s->N_user = N;
      for (int q = 0; q < 9; ++q) sup_s->user_lat[q] = cell[q];
      if ((rc = tm_alloc(ctx, (void**)&sup_s->d_xuser, sizeof(double) * 3 * (size_t)N))) {
        tm_system_destroy(sup_s);
        return rc;
      }
      *out = sup_s;
      return TM_OK;
    }
    // With plane spacings >= 2 * cutoff, every nonzero lattice vector is at
    // least 2 * cutoff long, so at most one image of an atom lies within the
    // cutoff of another, and a +-R cell search (R = ceil(cutoff / cell
    // spacing) <= n / 2) wraps at most once per axis and reaches each
    // (cell, image) at most once; the exact distance test keeps that image.
    s->periodic = true;
    // Coulomb grid: floor(h / size) cells per plane spacing, ~24 atoms per cell
    const double cs = std::max(2.0, cbrt(24.0 * std::fabs(vol) / N));
    for (int d = 0; d < 3; ++d) s->ee_dims[d] = std::max(1, std::min(4096, (int)floor(s->hpl[d] / cs)));
  }
  s->N_user = N;
  if (cell)
    for (int q = 0; q < 9; ++q) s->user_lat[q] = cell[q];
  SysLayout L;
  int rc = build_layout(s, N, nmol, Z, off, L);
  if (!rc) rc = system_alloc(s, N, nmol, L.Mpad, L.nchunk, L.ncell_cap, L.ecell_cap);
  if (!rc) rc = upload_layout(s, L);
  if (rc) {
    system_free(s);
    return rc;
  }
  *out = s;
  return TM_OK;
}

// Open-boundary system with room for up to N_cap atoms in nmol_cap molecules
// and no atoms yet (serving batches; layouts come from tm_system_relayout).
int tm_system_create_capacity(tm_model* m, int N_cap, int nmol_cap, tm_system** out) {
  *out = nullptr;
  tm_ctx* ctx = m->ctx;
  if (!m->final_) return tm_fail(ctx, TM_E_STATE, "model weights are not finalized");
  if (N_cap <= 0 || nmol_cap <= 0 || N_cap >= (1 << 27)) return tm_fail(ctx, TM_E_ARG, "capacity");
  tm_system* s = new tm_system();
  s->model = m;
  s->ctx = ctx;
  const int nele = m->k.nele;
  const int Mpad_cap = ((N_cap + TM_BM - 1) / TM_BM + nele) * TM_BM;
  const int nchunk_cap = N_cap / TM_CHUNK + nmol_cap;
  const int rc = system_alloc(s, N_cap, nmol_cap, Mpad_cap, nchunk_cap, 2 * N_cap + 64 * nmol_cap,
                              N_cap / 8 + 8 * nmol_cap);
  if (rc) {
    system_free(s);
    return rc;
  }
  *out = s;
  return TM_OK;
}

int tm_system_relayout(tm_system* s, int N, int nmol, const int32_t* Z, const int64_t* off) {
  if (s->periodic) return tm_fail(s->ctx, TM_E_UNSUPPORTED, "relayout of a periodic system");
  SysLayout L;
  int rc = build_layout(s, N, nmol, Z, off, L);
  if (!rc) rc = upload_layout(s, L);
  return rc;
}

static void system_free(tm_system* s) {
  tm_ctx* ctx = s->ctx;
  // sizes are not needed by cudaFreeAsync; budget accounting uses s->bytes
  void* ptrs[] = {s->row_of_atom, s->atom_of_row, s->tile_elem, s->d_Z, s->d_elem, s->d_mol,
                  s->d_off, s->d_x, s->d_xhi, s->d_xlo, s->d_x_at_build, s->d_grid, s->d_ncell, s->d_ncell_m, s->d_need,
                  s->d_chunk, s->d_mol_chunk, s->d_part, s->d_cbox,
                  s->d_egrid, s->d_encell, s->d_encell_m, s->d_ecell_cnt, s->d_ecell_start,
                  s->d_ecell_atoms, s->d_ecell_of_atom, s->d_epos, s->d_exhi, s->d_exlo, s->d_sort_tmp, s->d_scan_tmp, s->d_sort_tmp2, s->d_scan_tmp2, s->d_ccnt, s->d_cand, s->d_need_c, s->d_disp,
                  s->d_cacc, s->d_eblk, s->d_neblk,
                  s->d_cell_cnt, s->d_cell_start, s->d_cell_atoms, s->d_cell_of_atom, s->d_cnt_r,
                  s->d_cnt_a, s->d_nbr_r, s->d_nbr_a, s->d_rev_r, s->d_rev_a, s->d_sr, s->d_va,
                  s->dEdG, s->epart, s->d_Eatom, s->d_qraw, s->d_q, s->d_dEdq, s->d_fself,
                  s->d_fcv, s->d_ecv, s->d_F, s->d_mol_E, s->d_mol_aux, s->d_xuser, s->kink_g2, s->kink_h2[0],
                  s->kink_h2[1], s->kink_mask, s->kink_count, s->kink_rows, s->kink_nrows,
                  s->relu_mask};
  for (void* p : ptrs)
    if (p) cudaFreeAsync(p, ctx->stream);
  for (int h = 0; h < 2; ++h) {
    if (h == 1 && s->G[1] == s->G[0]) break;
    void* q[] = {s->G[h], s->H1[h], s->H2[h], s->G3[h]};
    for (void* p : q)
      if (p) cudaFreeAsync(p, ctx->stream);
  }
  ctx->in_use -= std::min(ctx->in_use, s->bytes);
  cudaStreamSynchronize(ctx->stream);
  if (s->h_stage) cudaFreeHost(s->h_stage);
  if (s->stage_ev) cudaEventDestroy(s->stage_ev);
  s->h_stage = nullptr;
  s->stage_ev = nullptr;
  delete s;
}

extern "C" int tm_system_destroy(tm_system* s) {
  if (s) system_free(s);
  return TM_OK;
}

// Small cells: copy c = (c0 r1 + c1) r2 + c2 of atom a at x_a + c0 a0 + c1 a1
// + c2 a2, formed left to right as the reference's tessellation forms images
// (Periodic.py:170-173).
__global__ void k_replicate(const double* __restrict__ xu, double* __restrict__ X, int N, int r1,
                            int r2, int K, const tm_mat3 lat) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= N * K) return;
  const int c = q / N, a = q - c * N;
  const int c0 = c / (r1 * r2), c1 = (c / r2) % r1, c2 = c % r2;
  for (int d = 0; d < 3; ++d)
    X[3 * q + d] = tm_image_coord(xu[3 * a + d], c0, c1, c2, lat.v[d], lat.v[3 + d], lat.v[6 + d]);
}

// per-cell totals of a replicated system: the supercell's energies and dipole / K
__global__ void k_per_cell(double* __restrict__ mol_E, double* __restrict__ mol_aux, double invK) {
  const int t = threadIdx.x;
  if (t < 4) mol_E[t] *= invK;
  if (t >= 4 && t < 7) mol_aux[2 + t - 4] *= invK;
}

static int user_natoms(const tm_system* s) { return s->K > 1 ? s->N_user : s->N; }

// positions of a replicated system: the caller's cell into d_xuser, then the copies
static int replicate_positions(tm_system* s, const double* x, cudaMemcpyKind kind) {
  tm_ctx* ctx = s->ctx;
  int rc = tm_cuda_check(ctx, cudaMemcpyAsync(s->d_xuser, x, sizeof(double) * 3 * s->N_user, kind,
                                              ctx->stream), "positions");
  if (rc) return rc;
  k_replicate<<<tm_div_up(s->N, 256), 256, 0, ctx->stream>>>(s->d_xuser, s->d_x, s->N_user, s->rep[1],
                                                             s->rep[2], s->K, tm_mat3_of(s->user_lat));
  ctx->launches++;
  return tm_cuda_check(ctx, cudaGetLastError(), "replicate");
}

extern "C" int tm_system_natoms(const tm_system* s) { return s ? user_natoms(s) : -1; }

extern "C" int tm_system_set_positions(tm_system* s, const double* x, int on_device) {
  if (!s || !x) return TM_E_ARG;
  tm_ctx* ctx = s->ctx;
  s->nlist_valid = false;
  if (s->K > 1)
    return replicate_positions(s, x, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
  return tm_cuda_check(ctx, cudaMemcpyAsync(s->d_x, x, sizeof(double) * 3 * s->N,
                                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                            ctx->stream),
                       "positions");
}

extern "C" int tm_system_get_positions(tm_system* s, double* x, int on_device) {
  if (!s || !x) return TM_E_ARG;
  tm_ctx* ctx = s->ctx;
  int rc = tm_cuda_check(ctx, cudaMemcpyAsync(x, s->d_x, sizeof(double) * 3 * user_natoms(s),
                                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                              ctx->stream),
                         "positions");
  if (rc) return rc;
  return tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "positions");
}

extern "C" int tm_system_build_nlist(tm_system* s) {
  if (!s) return TM_E_ARG;
  for (int attempt = 0; attempt < 3; ++attempt) {
    int rc = tm_launch_nlist(s);
    if (rc) return rc;
    bool grew = false;
    if ((rc = tm_nlist_grow(s, &grew))) return rc;
    if (!grew) return tm_sync_status(s->ctx, "build_nlist");
  }
  return tm_fail(s->ctx, TM_E_CAPACITY, "neighbour rows could not be grown");
}

extern "C" int tm_system_nlist_counts(tm_system* s, int64_t counts[4]) {
  if (!s || !counts) return TM_E_ARG;
  if (s->K > 1)
    return tm_fail(s->ctx, TM_E_UNSUPPORTED, "list export of a cell below twice the cutoff");
  if (!s->nlist_valid) return tm_fail(s->ctx, TM_E_STATE, "neighbour lists not built");
  return tm_count_nlist(s, counts);
}

extern "C" int tm_system_export_nlist(tm_system* s, int64_t* radp, int64_t* angt, int64_t* mil_j,
                                      int64_t* mil_jk, int on_device) {
  if (!s) return TM_E_ARG;
  if (s->K > 1)
    return tm_fail(s->ctx, TM_E_UNSUPPORTED, "list export of a cell below twice the cutoff");
  tm_ctx* ctx = s->ctx;
  if (!s->nlist_valid) return tm_fail(ctx, TM_E_STATE, "neighbour lists not built");
  int64_t c[4];
  int rc = tm_count_nlist(s, c);
  if (rc) return rc;
  const int64_t P = c[0], T = c[1];
  int64_t* dst[4] = {radp, angt, mil_j, mil_jk};
  const int64_t sz[4] = {P * 4, T * 5, P * 4, T * 4};
  int64_t* dev[4] = {nullptr, nullptr, nullptr, nullptr};
  for (int q = 0; q < 4; ++q) {
    if (!dst[q]) continue;
    if (on_device) { dev[q] = dst[q]; continue; }
    if ((rc = tm_alloc(ctx, (void**)&dev[q], sizeof(int64_t) * (size_t)std::max<int64_t>(sz[q], 1))))
      return rc;
  }
  rc = tm_launch_export_nlist(s, dev[0], dev[1], dev[2], dev[3], P, T);
  for (int q = 0; q < 4; ++q) {
    if (!dst[q] || on_device) continue;
    if (!rc && sz[q] > 0)
      rc = tm_cuda_check(ctx, cudaMemcpyAsync(dst[q], dev[q], sizeof(int64_t) * sz[q], cudaMemcpyDeviceToHost, ctx->stream), "export");
    tm_free(ctx, dev[q], sizeof(int64_t) * (size_t)std::max<int64_t>(sz[q], 1));
  }
  if (!rc) rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "export");
  return rc;
}

extern "C" int tm_system_export_ee(tm_system* s, int64_t* eep, int64_t cap, int on_device) {
  if (!s || !eep) return TM_E_ARG;
  if (s->K > 1)
    return tm_fail(s->ctx, TM_E_UNSUPPORTED, "list export of a cell below twice the cutoff");
  tm_ctx* ctx = s->ctx;
  if (!s->nlist_valid) return tm_fail(ctx, TM_E_STATE, "neighbour lists not built");
  if (on_device) return tm_launch_export_ee(s, eep, cap);
  int64_t* dev = nullptr;
  int rc = tm_alloc(ctx, (void**)&dev, sizeof(int64_t) * 3 * (size_t)std::max<int64_t>(cap, 1));
  if (rc) return rc;
  rc = tm_launch_export_ee(s, dev, cap);
  if (!rc) {
    int64_t n = 0;
    rc = tm_count_ee(s, &n);
    if (!rc && n > 0)
      rc = tm_cuda_check(ctx, cudaMemcpyAsync(eep, dev, sizeof(int64_t) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream), "ee");
    if (!rc) rc = tm_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "ee");
  }
  tm_free(ctx, dev, sizeof(int64_t) * 3 * (size_t)std::max<int64_t>(cap, 1));
  return rc;
}

// Device-side pipeline of one energy(+force) evaluation; no host sync unless
// the neighbour lists have to be (re)built.
// ev (optional, 7 events): recorded on the ctx stream before the lists, the
// descriptors, the network forward, the network backward, the pair terms, the
// adjoint, and at the end.
static int energy_force_pipeline(tm_system* s, unsigned flags, cudaEvent_t* ev) {
  int rc;
  cudaStream_t st = s->ctx->stream;
  const bool force = !(flags & TM_F_ENERGY_ONLY);
  if (ev) cudaEventRecord(ev[0], st);
  if (s->skin > 0.0 && s->cand_valid && !s->cand_rebuild) {
    if ((rc = tm_launch_nlist_filter(s))) return rc;      // exact rows from the candidates
  } else if (!(flags & TM_F_REUSE_NLIST) || !s->nlist_valid) {
    if ((rc = tm_launch_nlist(s))) return rc;
  } else {
    if ((rc = tm_launch_positions(s))) return rc;
  }
  if (ev) cudaEventRecord(ev[1], st);
  if ((rc = tm_launch_descriptors(s))) return rc;
  if (ev) cudaEventRecord(ev[2], st);
  if (ev) {
    // stage timing: one stream, in order
    if ((rc = tm_launch_mlp(s, false))) return rc;
    cudaEventRecord(ev[3], st);
    if (force && (rc = tm_launch_mlp_backward_only(s))) return rc;
    cudaEventRecord(ev[4], st);
    if ((rc = tm_launch_mlp_finish(s))) return rc;
    if ((rc = tm_launch_coulomb(s, flags))) return rc;
    cudaEventRecord(ev[5], st);
  } else {
    if ((rc = tm_launch_mlp(s, false))) return rc;
    if ((rc = tm_launch_mlp_finish(s))) return rc;
    if (force) {
      // The backward pass of both networks needs no pair term (dE/dq enters
      // in the adjoint), so the pair terms run on the second stream beside it.
      // A GEMM CTA takes 225 KB of the SM's 228 KB of shared memory, so the
      // two kernels do not share an SM. Submitted first, the pair kernel fills
      // the GEMM's idle SMs and the launch gaps at both ends, and the GEMMs
      // then start on SMs that it has drained. Submitted second (measured),
      // its blocks slip in between the three GEMM launches and delay the
      // persistent CTAs of the next one.
      tm_ctx* ctx = s->ctx;
      cudaEventRecord(ctx->ev_fork, st);
      cudaStreamWaitEvent(ctx->aux, ctx->ev_fork, 0);
      ctx->stream = ctx->aux;
      rc = tm_launch_coulomb(s, flags);
      ctx->stream = st;
      cudaEventRecord(ctx->ev_join, ctx->aux);
      if (!rc) rc = tm_launch_mlp_backward_only(s);
      cudaStreamWaitEvent(st, ctx->ev_join, 0);   // joined even after an error
      if (rc) return rc;
    } else if ((rc = tm_launch_coulomb(s, flags))) {
      return rc;
    }
  }
  if (force && (rc = tm_launch_adjoint(s, flags))) return rc;
  if (ev) cudaEventRecord(ev[6], st);
  return TM_OK;
}

int tm_energy_force_device(tm_system* s, unsigned flags) {
  return energy_force_pipeline(s, flags, nullptr);
}

extern "C" int tm_energy_force_profile(tm_system* s, unsigned flags, float* stage_ms) {
  if (!s || !stage_ms) return TM_E_ARG;
  tm_ctx* ctx = s->ctx;
  cudaEvent_t ev[7];
  for (auto& e : ev) cudaEventCreate(&e);
  int rc = energy_force_pipeline(s, flags & ~(unsigned)TM_F_DEVICE_IO, ev);
  if (!rc) rc = tm_cuda_check(ctx, cudaEventSynchronize(ev[6]), "profile");
  if (!rc) {
    for (int q = 0; q < 6; ++q) cudaEventElapsedTime(&stage_ms[q], ev[q], ev[q + 1]);
    cudaEventElapsedTime(&stage_ms[6], ev[0], ev[6]);
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (!rc) rc = tm_sync_status(ctx, "profile");
  return rc;
}

extern "C" int tm_energy_force(tm_system* s, const double* x, unsigned flags, double* E_out,
                               double* F_out, double* q_out, double* dipole_out, double* Eatom_out) {
  if (!s) return TM_E_ARG;
  tm_ctx* ctx = s->ctx;
  const bool dev = flags & TM_F_DEVICE_IO;
  int rc;
  if (s->K > 1 && (flags & TM_F_REFERENCE_PERIODIC_FORCE))
    return tm_fail(ctx, TM_E_UNSUPPORTED, "the images-fixed force of a cell below twice the cutoff");
  if (x) {
    if (s->K > 1) {
      if ((rc = replicate_positions(s, x, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice)))
        return rc;
    } else if ((rc = tm_cuda_check(ctx, cudaMemcpyAsync(s->d_x, x, sizeof(double) * 3 * s->N,
                                                        dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                                        ctx->stream),
                                   "x"))) {
      return rc;
    }
    if (!(flags & TM_F_REUSE_NLIST)) s->nlist_valid = false;
  }
  for (int attempt = 0;; ++attempt) {
    if ((rc = tm_energy_force_device(s, flags))) return rc;
    bool grew = false;
    if ((rc = tm_nlist_grow(s, &grew))) return rc;
    if (!grew) break;
    if (attempt == 2) return tm_fail(ctx, TM_E_CAPACITY, "neighbour rows could not be grown");
  }
  const cudaMemcpyKind kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  cudaStream_t st = ctx->stream;
  // a replicated cell: copy 0's per-atom results, the supercell's totals / K
  const int Nu = user_natoms(s);
  if (s->K > 1) {
    k_per_cell<<<1, 32, 0, st>>>(s->d_mol_E, s->d_mol_aux, 1.0 / s->K);
    ctx->launches++;
  }
  if (E_out) cudaMemcpyAsync(E_out, s->d_mol_E, sizeof(double) * 4 * s->nmol, kind, st);
  if (F_out && !(flags & TM_F_ENERGY_ONLY)) cudaMemcpyAsync(F_out, s->d_F, sizeof(double) * 3 * Nu, kind, st);
  if (Eatom_out) cudaMemcpyAsync(Eatom_out, s->d_Eatom, sizeof(double) * Nu, kind, st);
  if (q_out || dipole_out) {
    // q (float) and dipole (aux[2..4]) are converted on the host side
    std::vector<float> qf(Nu);
    std::vector<double> aux((size_t)8 * s->nmol);
    cudaMemcpyAsync(qf.data(), s->d_q, sizeof(float) * Nu, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(aux.data(), s->d_mol_aux, sizeof(double) * 8 * s->nmol, cudaMemcpyDeviceToHost, st);
    if ((rc = tm_sync_status(ctx, "energy_force"))) return rc;
    std::vector<double> qd(Nu), dip((size_t)3 * s->nmol);
    for (int i = 0; i < Nu; ++i) qd[i] = qf[i];
    for (int m = 0; m < s->nmol; ++m)
      for (int d = 0; d < 3; ++d) dip[3 * m + d] = aux[8 * m + 2 + d];
    if (q_out) cudaMemcpy(q_out, qd.data(), sizeof(double) * Nu, dev ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost);
    if (dipole_out) cudaMemcpy(dipole_out, dip.data(), sizeof(double) * 3 * s->nmol, dev ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost);
  }
  return tm_sync_status(ctx, "energy_force");
}

// ---------------------------------------------------------------------------
// diagnostics
// ---------------------------------------------------------------------------
extern "C" int tm_selftest_gemm(tm_ctx* ctx, int prec, int M, int N, int K, const float* A,
                                const float* B, float* C) {
  if (!ctx || !A || !B || !C) return TM_E_ARG;
  if (prec != TM_PREC_FP32 && prec != TM_PREC_BF16) return tm_fail(ctx, TM_E_ARG, "precision");
  return tm_gemm_selftest(ctx, prec, M, N, K, A, B, C);
}

extern "C" int tm_selftest_gemm_timeout(tm_ctx* ctx, int prec, int64_t wait_cycles) {
  if (!ctx || wait_cycles <= 0 || wait_cycles > (1LL << 28)) return TM_E_ARG;
  if (prec != TM_PREC_FP32 && prec != TM_PREC_BF16) return tm_fail(ctx, TM_E_ARG, "precision");
  const int M = 256, N = 256, K = 256;
  std::vector<float> A((size_t)M * K, 0.5f), B((size_t)N * K, 0.25f), C((size_t)M * N, 0.f);
  // the second operand stage of every CTA is withheld: the MMA issuer's wait on it
  // runs out, then the producer's and the epilogue's waits do
  return tm_gemm_selftest(ctx, prec, M, N, K, A.data(), B.data(), C.data(), wait_cycles, 1);
}

extern "C" int tm_system_layer_outputs(tm_system* s, int layer, float* out) {
  if (!s || !out) return TM_E_ARG;
  tm_ctx* ctx = s->ctx;
  const tm_model* m = s->model;
  const int L = m->nlayer, H = m->H;
  if (layer < 0 || layer >= L) return tm_fail(ctx, TM_E_ARG, "layer index");
  const int width = m->desc.hidden[layer];
  void* const* buf = layer == L - 1 ? s->G3 : (layer == 0 ? s->H1 : s->H2);
  const size_t n = (size_t)2 * s->Mpad * H;
  const bool split = m->desc.precision == TM_PREC_FP32;
  // FP32 relu: the last layer holds act'(z) in {0, 1}, one plane
  const bool one_plane = split && layer == L - 1 && m->w_bwd_fold[0];
  std::vector<float> hi(n), lo(split ? n : 0);
  std::vector<uint16_t> b16(split ? 0 : n);
  int rc;
  if (split) {
    if ((rc = tm_cuda_check(ctx, cudaMemcpyAsync(hi.data(), buf[0], n * 4, cudaMemcpyDeviceToHost, ctx->stream), "layer outputs")) ||
        (rc = tm_cuda_check(ctx, cudaMemcpyAsync(lo.data(), buf[1], n * 4, cudaMemcpyDeviceToHost, ctx->stream), "layer outputs")))
      return rc;
  } else if ((rc = tm_cuda_check(ctx, cudaMemcpyAsync(b16.data(), buf[0], n * 2, cudaMemcpyDeviceToHost, ctx->stream), "layer outputs"))) {
    return rc;
  }
  if ((rc = tm_sync_status(ctx, "layer outputs"))) return rc;
  const int Nu = user_natoms(s);
  for (int net = 0; net < 2; ++net)
    for (int i = 0; i < Nu; ++i) {
      const size_t src = ((size_t)net * s->Mpad + s->row_of_atom_h[i]) * H;
      float* dst = out + ((size_t)net * Nu + i) * width;
      for (int c = 0; c < width; ++c) {
        if (split) {
          dst[c] = one_plane ? hi[src + c] : hi[src + c] + lo[src + c];
        } else {
          const uint32_t u = (uint32_t)b16[src + c] << 16;
          memcpy(&dst[c], &u, 4);
        }
      }
    }
  return TM_OK;
}

extern "C" int tm_system_profile_layers(tm_system* s, float* ms) {
  if (!s || !ms) return TM_E_ARG;
  if (!s->nlist_valid) return tm_fail(s->ctx, TM_E_STATE, "evaluate the system first");
  return tm_profile_layers(s, ms);
}

extern "C" int tm_system_refined_units(tm_system* s, int64_t* n) {
  if (!s || !n) return TM_E_ARG;
  *n = 0;
  if (!s->kink_count) return TM_OK;
  unsigned long long c = 0;
  int rc = tm_cuda_check(s->ctx, cudaMemcpyAsync(&c, s->kink_count, sizeof(c), cudaMemcpyDeviceToHost,
                                                 s->ctx->stream), "refined units");
  if (!rc) rc = tm_cuda_check(s->ctx, cudaStreamSynchronize(s->ctx->stream), "refined units");
  *n = (int64_t)c;
  return rc;
}

int tm_launch_descriptors_f32(tm_system* s, float* out);

extern "C" int tm_system_descriptors(tm_system* s, float* G_out) {
  if (!s || !G_out) return TM_E_ARG;
  tm_ctx* ctx = s->ctx;
  int rc;
  for (int attempt = 0; attempt < 3; ++attempt) {
    if (!s->nlist_valid) {
      if ((rc = tm_launch_nlist(s))) return rc;
      bool grew = false;
      if ((rc = tm_nlist_grow(s, &grew))) return rc;
      if (grew) continue;
    }
    break;
  }
  const int Dp = s->model->k.Dp, D = s->model->k.D;
  float* dev = nullptr;
  if ((rc = tm_alloc(ctx, (void**)&dev, sizeof(float) * (size_t)s->Mpad * Dp))) return rc;
  cudaMemsetAsync(dev, 0, sizeof(float) * (size_t)s->Mpad * Dp, ctx->stream);
  if (!(rc = tm_launch_descriptors_f32(s, dev))) {
    std::vector<float> rows((size_t)s->Mpad * Dp);
    rc = tm_cuda_check(ctx, cudaMemcpyAsync(rows.data(), dev, rows.size() * 4, cudaMemcpyDeviceToHost, ctx->stream), "G");
    if (!rc) rc = tm_sync_status(ctx, "descriptors");
    if (!rc)
      for (int i = 0; i < user_natoms(s); ++i)
        memcpy(G_out + (size_t)i * D, rows.data() + (size_t)s->row_of_atom_h[i] * Dp, sizeof(float) * D);
  }
  tm_free(ctx, dev, sizeof(float) * (size_t)s->Mpad * Dp);
  return rc;
}
