// K6 grid correction + image accumulation, the per-pixel n-1 table, the
// prediction pre-correction and output permutation, and K7 gains + collapse.
#include <cmath>
#include <vector>

#include "polarization.cuh"
#include "screen.cuh"
#include "wgpu_internal.h"

namespace wgpu {

namespace {

constexpr int kThreads = 256;

unsigned blocks_for(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// Row of sample e (n samples, n_chan per row): 32-bit division when n < 2^32
// (the common case; it needs no FP64), 64-bit otherwise.
__device__ __forceinline__ int64_t row_of(int64_t e, int64_t n, int64_t n_chan) {
  if (n < (int64_t)0xFFFFFFFFll) return (int64_t)((uint32_t)e / (uint32_t)n_chan);
  return e / n_chan;
}

// n - 1 - c_n per trimmed pixel, FP64.  Pixel (x, y) at l = (width/2 - x) dl +
// l_shift, m = (y - height/2) dm + m_shift, n - 1 := 0 beyond the horizon
// (gridding/directmsgridder.cpp:205-229).
__global__ void nu_table_kernel(DevPlan p, double *nu_w) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)p.width * p.height) return;
  const int x = (int)(i % p.width), y = (int)(i / p.width);
  const double l = (double)(p.width / 2 - x) * p.dl + p.l_shift;
  const double m = (double)(y - p.height / 2) * p.dm + p.m_shift;
  const double r2 = l * l + m * m;
  const double nm1 = r2 >= 1.0 ? 0.0 : -r2 / (sqrt(1.0 - r2) + 1.0);
  nu_w[i] = nm1 - p.nm1_center;
}

// w-screen terms per pixel (screen.cuh): the screen of plane q, w_q = w0 +
// q dw, is exp(-+2 pi i w_q nu), the per-plane screen of ducc0's w-gridding
// behind ms2dirty / dirty2ms (wgridder/gridder_simple.h:216-225), whose
// argument is formed in FP64.
__global__ void screen_table_kernel(DevPlan p, const double *nu_w, ScreenTable scr) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)p.width * p.height) return;
  const ScreenTerms t = screen_terms(p.w0, p.dw, nu_w[i]);
  scr.a[i] = t.a;
  scr.k[i] = t.k;
  scr.r[i] = t.r;
}

// Grid-correction tables: thread t < width gives cx[t] = 1 / psihat((width/2 -
// t) / nu), the next height threads cy[y] = 1 / psihat((y - height/2) / nv),
// psihat(f) = W sum_i g_i cos(pi f W z_i) over the planner's quadrature (the
// same sum as es_fourier, in FP64); the first 2 kCorrGlNodes threads also copy
// the w-factor nodes.
struct CorrQuad {
  double z[kEsQuadNodes], g[kEsQuadNodes];
  float gl[2 * kCorrGlNodes];
};

__global__ void correction_tables_kernel(const CorrQuad q, int width, int height, int nu, int nv,
                                         int support, float *cx, float *cy, float *gl) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 2 * kCorrGlNodes) gl[t] = q.gl[t];
  if (t >= width + height) return;
  const double f = t < width ? (double)(width / 2 - t) / (double)nu
                             : (double)(t - width - height / 2) / (double)nv;
  double acc = 0.0;
  for (int i = 0; i < kEsQuadNodes; ++i) acc += q.g[i] * cos(M_PI * f * support * q.z[i]);
  const float v = (float)(1.0 / (support * acc));
  if (t < width)
    cx[t] = v;
  else
    cy[t - width] = v;
}

// 1 / psihat(dw * nu) by Gauss-Legendre quadrature over the positive half:
// psihat(f) = W * sum_q g_q cos(pi f W z_q), g_q = w_q phi(z_q).
__device__ __forceinline__ float w_correction(const DevPlan &p, double nu,
                                              const float *gl_zw, int n_gl) {
  if (p.n_planes == 1) return 1.0f;
  const float a = (float)(M_PI * p.dw * nu * p.support);
  float acc = 0.0f;
  for (int q = 0; q < n_gl; ++q) acc += gl_zw[2 * q + 1] * cosf(a * gl_zw[2 * q]);
  return 1.0f / ((float)p.support * acc);
}

// The w correction of every pixel, once per plan (finalize_add_kernel and
// precorrect_kernel read it).
__global__ void wcorr_table_kernel(DevPlan p, const double *nu_w, const float *gl_zw, int n_gl,
                                   float *wcorr) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)p.width * p.height) return;
  wcorr[i] = w_correction(p, nu_w[i], gl_zw, n_gl);
}

template <typename NumT>
__global__ void finalize_add_kernel(DevPlan p, const float2 *acc,
                                    const float *wcorr, const float *cx,
                                    const float *cy, NumT *img) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)p.width * p.height) return;
  const int x = (int)(i % p.width), y = (int)(i / p.width);
  const float2 a = acc[i];
  const float v = (a.x - a.y) * cx[x] * cy[y] * wcorr[i];
  img[i] += (NumT)v;
}

template <typename NumT>
__global__ void precorrect_kernel(DevPlan p, const NumT *img, const float *wcorr,
                                  const float *cx, const float *cy, float *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)p.width * p.height) return;
  const int x = (int)(i % p.width), y = (int)(i / p.width);
  const float v = (float)img[i];
  out[i] = v == 0.0f ? 0.0f : v * cx[x] * cy[y] * wcorr[i];
}

// The degridded sums (already times the conjugate of each record's phase
// factor) back into sample order.
__global__ void unpermute_predict_kernel(const uint32_t *perm, const float2 *acc, int64_t n,
                                         float2 *vis) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  vis[__ldg(perm + s)] = acc[s];
}

// ---- K7: conjugated gains (visibilitymodifier.h:378-401) + collapse -------
__global__ void apply_gains_kernel(int mode, int n_pol, int64_t n_rows,
                                   int64_t n_chan, const float2 *vis_in,
                                   const uint64_t *ant_pairs,
                                   const uint64_t *time_offsets,
                                   const float2 *sol, int nparms,
                                   int64_t n_times, int64_t n_ant,
                                   int polarization, float2 *out,
                                   int *err_flag) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_rows * n_chan) return;
  const int64_t r = row_of(e, n_rows * n_chan, n_chan), ch = e - r * n_chan;
  const uint64_t a1 = ant_pairs[2 * r], a2 = ant_pairs[2 * r + 1];
  const uint64_t t = time_offsets[r];
  if (a1 >= (uint64_t)n_ant || a2 >= (uint64_t)n_ant || t >= (uint64_t)n_times) {
    // out-of-range index: record it and leave the visibility out (zero)
    atomicOr(err_flag, 1);
    out[e] = make_float2(0.f, 0.f);
    return;
  }
  const int64_t off = ((int64_t)t * n_chan + ch) * n_ant * nparms;
  float2 g1[4], g2[4];
  if (nparms == 2) {
    g1[0] = sol[off + a1 * 2]; g1[1] = make_float2(0.f, 0.f);
    g1[2] = make_float2(0.f, 0.f); g1[3] = sol[off + a1 * 2 + 1];
    g2[0] = sol[off + a2 * 2]; g2[1] = make_float2(0.f, 0.f);
    g2[2] = make_float2(0.f, 0.f); g2[3] = sol[off + a2 * 2 + 1];
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      g1[k] = sol[off + a1 * 4 + k];
      g2[k] = sol[off + a2 * 4 + k];
    }
  }
  float2 v[4];
  for (int k = 0; k < n_pol; ++k) v[k] = vis_in[e * n_pol + k];
  float2 res;
  switch (mode) {
    case 0: res = cm(cm(cj(g1[0]), v[0]), g2[0]); break;
    case 1: res = cm(cm(cj(g1[3]), v[0]), g2[3]); break;
    case 2: {
      float2 dd = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < 4; ++k) dd = ca(dd, cm(g2[k], cj(g1[k])));
      res = cm(v[0], cs(dd, 0.5f));
      break;
    }
    case 3: {
      // second component uses the updated first one, as in
      // visibilitymodifier.h:393-396
      const float2 v0 = ca(cm(cm(cj(g1[0]), v[0]), g2[0]), cm(cm(cj(g1[2]), v[1]), g2[2]));
      const float2 v1 = ca(cm(cm(cj(g1[3]), v[1]), g2[3]), cm(cm(cj(g1[1]), v0), g2[1]));
      res = ca(v0, v1);  // msgridderdata.h:41-45 collapse: v0 + v1
      break;
    }
    default: {
      float2 t1[4], t2[4];
      herm_mul(g1, v, t1);
      mat_mul(t1, g2, t2);
      res = collapse4(t2, polarization);
      break;
    }
  }
  out[e] = res;
}

// ---- prediction write-back: forward gains (visibilitymodifier.h:345-370) ----
// r = a b^H (row-major 2x2)
__device__ __forceinline__ void mul_herm(const float2 *a, const float2 *b, float2 *r) {
  r[0] = ca(cm(a[0], cj(b[0])), cm(a[1], cj(b[1])));
  r[1] = ca(cm(a[0], cj(b[2])), cm(a[1], cj(b[3])));
  r[2] = ca(cm(a[2], cj(b[0])), cm(a[3], cj(b[1])));
  r[3] = ca(cm(a[2], cj(b[2])), cm(a[3], cj(b[3])));
}

// Predicted [row][chan] values -> [row][chan][n_pol] instrumental
// visibilities: expanded to the correlations (msgridderdata.h:180-202) and
// multiplied by the forward gains of the row's antennas
// (visibilitymodifier.cpp:196-228, ApplyGain).
__global__ void forward_gains_kernel(int mode, int n_pol, int64_t n_rows, int64_t n_chan,
                                     const float2 *vis_in, const uint64_t *ant_pairs,
                                     const uint64_t *time_offsets, const float2 *sol, int nparms,
                                     int64_t n_times, int64_t n_ant, int polarization,
                                     float2 *out, int *err_flag) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_rows * n_chan) return;
  const int64_t r = row_of(e, n_rows * n_chan, n_chan), ch = e - r * n_chan;
  float2 *o = out + e * n_pol;
  const uint64_t a1 = ant_pairs[2 * r], a2 = ant_pairs[2 * r + 1];
  const uint64_t t = time_offsets[r];
  if (a1 >= (uint64_t)n_ant || a2 >= (uint64_t)n_ant || t >= (uint64_t)n_times) {
    atomicOr(err_flag, 1);
    for (int k = 0; k < n_pol; ++k) o[k] = make_float2(0.f, 0.f);
    return;
  }
  const int64_t off = ((int64_t)t * n_chan + ch) * n_ant * nparms;
  float2 g1[4], g2[4];
  if (nparms == 2) {
    g1[0] = sol[off + a1 * 2]; g1[1] = make_float2(0.f, 0.f);
    g1[2] = make_float2(0.f, 0.f); g1[3] = sol[off + a1 * 2 + 1];
    g2[0] = sol[off + a2 * 2]; g2[1] = make_float2(0.f, 0.f);
    g2[2] = make_float2(0.f, 0.f); g2[3] = sol[off + a2 * 2 + 1];
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      g1[k] = sol[off + a1 * 4 + k];
      g2[k] = sol[off + a2 * 4 + k];
    }
  }
  const float2 s = vis_in[e];
  switch (mode) {
    case 0: o[0] = cm(cm(g1[0], s), cj(g2[0])); break;
    case 1: o[0] = cm(cm(g1[3], s), cj(g2[3])); break;
    case 2: {
      float2 dd = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < 4; ++k) dd = ca(dd, cm(g1[k], cj(g2[k])));
      o[0] = cm(s, cs(dd, 0.5f));
      break;
    }
    case 3: {
      // both correlations hold s (ExpandData<2>); the second uses the updated
      // first one, as ApplyGain does (visibilitymodifier.h:359-362)
      const float2 v0 = ca(cm(cm(g1[0], s), cj(g2[0])), cm(cm(g1[1], s), cj(g2[1])));
      const float2 v1 = ca(cm(cm(g1[3], s), cj(g2[3])), cm(cm(g1[2], v0), cj(g2[2])));
      o[0] = v0;
      o[1] = v1;
      break;
    }
    default: {
      float2 v[4], t1[4], t2[4];
      expand4(s, polarization, v);
      mat_mul(g1, v, t1);
      mul_herm(t1, g2, t2);
#pragma unroll
      for (int k = 0; k < 4; ++k) o[k] = t2[k];
      break;
    }
  }
}

}  // namespace

void launch_forward_gains(int mode, int n_pol, int64_t n_rows, int64_t n_chan,
                          const float2 *vis_in, const uint64_t *ant_pairs,
                          const uint64_t *time_offsets, const float2 *sol, int nparms,
                          int64_t n_times, int64_t n_ant, int polarization, float2 *out,
                          int *err_flag, cudaStream_t s) {
  const int64_t n = n_rows * n_chan;
  if (n <= 0) return;
  forward_gains_kernel<<<blocks_for(n), kThreads, 0, s>>>(mode, n_pol, n_rows, n_chan, vis_in,
                                                          ant_pairs, time_offsets, sol, nparms,
                                                          n_times, n_ant, polarization, out,
                                                          err_flag);
  check_launch("forward_gains_kernel");
}

// The Gauss-Legendre rule of 2 kCorrGlNodes points on [-1, 1] (positive
// half), computed once.
const std::vector<double> &corr_gl_rule() {
  static const std::vector<double> rule = [] {
    std::vector<double> r(2 * kCorrGlNodes);
    const int n = 2 * kCorrGlNodes;
    for (int i = 0; i < kCorrGlNodes; ++i) {
      double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
      for (int it = 0; it < 100; ++it) {
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; ++k) {
          const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
          p0 = p1;
          p1 = p2;
        }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        const double dz = p1 / dp;
        z -= dz;
        if (std::fabs(dz) < 1e-16) break;
      }
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      r[2 * i] = z;
      r[2 * i + 1] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    return r;
  }();
  return rule;
}

void launch_correction_tables(const wgpu_plan_t &plan, float *cx, float *cy, float *gl,
                              cudaStream_t s) {
  CorrQuad q;
  es_quadrature(plan.beta, q.z, q.g);
  const std::vector<double> &rule = corr_gl_rule();
  for (int i = 0; i < kCorrGlNodes; ++i) {
    q.gl[2 * i] = (float)rule[2 * i];
    q.gl[2 * i + 1] = (float)(rule[2 * i + 1] * es_kernel(plan.beta, rule[2 * i]));
  }
  const int n = (int)std::max<int64_t>(plan.width + plan.height, 2 * kCorrGlNodes);
  correction_tables_kernel<<<blocks_for(n), kThreads, 0, s>>>(
      q, (int)plan.width, (int)plan.height, (int)plan.nu, (int)plan.nv, (int)plan.support, cx, cy,
      gl);
  check_launch("correction_tables_kernel");
}

void launch_nu_table(const DevPlan &p, double *nu_w, cudaStream_t s) {
  const int64_t n = (int64_t)p.width * p.height;
  nu_table_kernel<<<blocks_for(n), kThreads, 0, s>>>(p, nu_w);
  check_launch("nu_table_kernel");
}

ScreenTable screen_table_at(void *buf, int64_t npix) {
  ScreenTable t;
  t.a = (uint32_t *)buf;
  t.k = t.a + npix;
  t.r = (float *)(t.k + npix);
  return t;
}

void launch_screen_table(const DevPlan &p, const double *nu_w, const ScreenTable &scr,
                         cudaStream_t s) {
  const int64_t n = (int64_t)p.width * p.height;
  screen_table_kernel<<<blocks_for(n), kThreads, 0, s>>>(p, nu_w, scr);
  check_launch("screen_table_kernel");
}

void launch_wcorr_table(const DevPlan &p, const double *nu_w, const float *gl_zw, int n_gl,
                        float *wcorr, cudaStream_t s) {
  const int64_t n = (int64_t)p.width * p.height;
  wcorr_table_kernel<<<blocks_for(n), kThreads, 0, s>>>(p, nu_w, gl_zw, n_gl, wcorr);
  check_launch("wcorr_table_kernel");
}

void launch_finalize_add(const DevPlan &p, const float2 *acc, const float *wcorr,
                         const float *cx, const float *cy, void *img, int precision_bytes,
                         cudaStream_t s) {
  const int64_t n = (int64_t)p.width * p.height;
  if (precision_bytes == 8)
    finalize_add_kernel<double><<<blocks_for(n), kThreads, 0, s>>>(p, acc, wcorr, cx, cy, (double *)img);
  else
    finalize_add_kernel<float><<<blocks_for(n), kThreads, 0, s>>>(p, acc, wcorr, cx, cy, (float *)img);
  check_launch("finalize_add_kernel");
}

void launch_precorrect(const DevPlan &p, const void *img, int precision_bytes,
                       const float *wcorr, const float *cx, const float *cy, float *img_corr,
                       cudaStream_t s) {
  const int64_t n = (int64_t)p.width * p.height;
  if (precision_bytes == 8)
    precorrect_kernel<double><<<blocks_for(n), kThreads, 0, s>>>(p, (const double *)img, wcorr, cx, cy, img_corr);
  else
    precorrect_kernel<float><<<blocks_for(n), kThreads, 0, s>>>(p, (const float *)img, wcorr, cx, cy, img_corr);
  check_launch("precorrect_kernel");
}

void launch_unpermute_predict(const uint32_t *perm, const float2 *acc, int64_t n, float2 *vis,
                              cudaStream_t s) {
  if (n <= 0) return;
  unpermute_predict_kernel<<<blocks_for(n), kThreads, 0, s>>>(perm, acc, n, vis);
  check_launch("unpermute_predict_kernel");
}

void launch_apply_gains(int mode, int n_pol, int64_t n_rows, int64_t n_chan,
                        const float2 *vis_in, const uint64_t *ant_pairs,
                        const uint64_t *time_offsets, const float2 *sol,
                        int nparms, int64_t n_times, int64_t n_ant,
                        int polarization, float2 *out, int *err_flag,
                        cudaStream_t s) {
  const int64_t n = n_rows * n_chan;
  if (n <= 0) return;
  apply_gains_kernel<<<blocks_for(n), kThreads, 0, s>>>(
      mode, n_pol, n_rows, n_chan, vis_in, ant_pairs, time_offsets, sol, nparms,
      n_times, n_ant, polarization, out, err_flag);
  check_launch("apply_gains_kernel");
}

}  // namespace wgpu

namespace wgpu {
namespace {
template <typename NumT>
__global__ void scale_kernel(NumT *img, int64_t n, double factor) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) img[i] = (NumT)(img[i] * factor);
}
}  // namespace

void launch_scale_image(void *img, int precision_bytes, int64_t n, double factor,
                        cudaStream_t s) {
  if (n <= 0) return;
  const unsigned b = (unsigned)((n + 255) / 256);
  if (precision_bytes == 8)
    scale_kernel<double><<<b, 256, 0, s>>>((double *)img, n, factor);
  else
    scale_kernel<float><<<b, 256, 0, s>>>((float *)img, n, factor);
  check_launch("scale_kernel");
}
}  // namespace wgpu

namespace wgpu {
namespace {
// Inversion records from stored prediction records: the geometry is kept and
// (re, im) becomes visibility x phase factor, the product the bucketing pass
// forms for inversion.
__global__ void restamp_kernel(const VisRecord *__restrict__ geom,
                               const uint32_t *__restrict__ perm,
                               const float2 *__restrict__ vis, int64_t n,
                               VisRecord *__restrict__ out) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const float4 a = __ldg(reinterpret_cast<const float4 *>(geom + s));
  const float4 b = __ldg(reinterpret_cast<const float4 *>(geom + s) + 1);
  const float2 v = __ldg(vis + perm[s]);
  // phase factor (a.x, a.y) = exp(-2 pi i theta)
  const float re = v.x * a.x - v.y * a.y;
  const float im = v.x * a.y + v.y * a.x;
  reinterpret_cast<float4 *>(out + s)[0] = make_float4(re, im, a.z, a.w);
  reinterpret_cast<float4 *>(out + s)[1] = b;
}
}  // namespace

void launch_restamp(const VisRecord *geom, const uint32_t *perm, const float2 *vis, int64_t n,
                    VisRecord *out, cudaStream_t s) {
  if (n <= 0) return;
  restamp_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(geom, perm, vis, n, out);
  check_launch("restamp_kernel");
}
}  // namespace wgpu
