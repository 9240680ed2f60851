/*
 * wgpu oracle -- TEST INFRASTRUCTURE ONLY (see wgpu_oracle.h for the parity
 * status of each part).  Compiled with -ffp-contract=off so that the bucketing
 * arithmetic rounds exactly like the GPU pass on every host architecture.
 */
#include "wgpu_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define C_LIGHT 299792458.0
#define TWO_PI 6.283185307179586476925286766559

/* ------------------------------------------------------------------------ */
/* Image geometry shared by the DFT and the gridder (directmsgridder.cpp).    */
/* ------------------------------------------------------------------------ */

/* l, m of trimmed pixel (x, y): directmsgridder.cpp:113-124 composed with the
 * output wrap of :70-82 gives l = (width/2 - x) dl + l_shift and
 * m = (y - height/2) dm + m_shift. */
static void pixel_lm(int64_t x, int64_t y, int64_t width, int64_t height,
                     double dl, double dm, double l_shift, double m_shift,
                     double *l, double *m) {
  *l = (double)(width / 2 - x) * dl + l_shift;
  *m = (double)(y - height / 2) * dm + m_shift;
}

/* n - 1 with the horizon rule of directmsgridder.cpp:218-221; written in the
 * cancellation-free form -r2 / (sqrt(1 - r2) + 1). */
static double pixel_nm1(double l, double m) {
  const double r2 = l * l + m * m;
  if (r2 >= 1.0) return 0.0;
  return -r2 / (sqrt(1.0 - r2) + 1.0);
}

static inline void sincos_turns(double t, double *s, double *c) {
  t -= rint(t);
  const double a = TWO_PI * t;
  *s = sin(a);
  *c = cos(a);
}

/* ------------------------------------------------------------------------ */
/* Direct FT                                                                  */
/* ------------------------------------------------------------------------ */

void oracle_dft_invert(size_t n_rows, size_t n_chan, const double *uvw,
                       const double *freq, const float *vis, size_t width,
                       size_t height, double dl, double dm, double l_shift,
                       double m_shift, const int64_t *pixels, size_t n_pixels,
                       int n_threads, double *out) {
  /* u, v, w in wavelengths for every non-zero visibility
   * (directmsgridder.cpp:166-176). */
  size_t n_vis = 0;
  for (size_t i = 0; i < n_rows * n_chan; ++i)
    if (vis[2 * i] != 0.0f || vis[2 * i + 1] != 0.0f) ++n_vis;
  double *buf = (double *)malloc(sizeof(double) * 5 * (n_vis + 1));
  size_t k = 0;
  for (size_t r = 0; r < n_rows; ++r)
    for (size_t c = 0; c < n_chan; ++c) {
      const size_t e = r * n_chan + c;
      if (vis[2 * e] == 0.0f && vis[2 * e + 1] == 0.0f) continue;
      const double inv_lambda = freq[c] / C_LIGHT;
      buf[5 * k + 0] = uvw[3 * r + 0] * inv_lambda;
      buf[5 * k + 1] = uvw[3 * r + 1] * inv_lambda;
      buf[5 * k + 2] = uvw[3 * r + 2] * inv_lambda;
      buf[5 * k + 3] = vis[2 * e];
      buf[5 * k + 4] = vis[2 * e + 1];
      ++k;
    }
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 4)
  for (size_t i = 0; i < n_pixels; ++i) {
    const int64_t p = pixels[i];
    const int64_t x = p % (int64_t)width, y = p / (int64_t)width;
    double l, m;
    pixel_lm(x, y, width, height, dl, dm, l_shift, m_shift, &l, &m);
    const double nm1 = pixel_nm1(l, m);
    double acc = 0.0;
    for (size_t j = 0; j < n_vis; ++j) {
      const double *b = buf + 5 * j;
      double s, c;
      sincos_turns(b[0] * l + b[1] * m + b[2] * nm1, &s, &c);
      /* Re(V exp(-2 pi i t)) (directmsgridder.cpp:127-129) */
      acc += b[3] * c + b[4] * s;
    }
    out[i] = acc;
  }
  free(buf);
}

void oracle_dft_predict(size_t n_rows, size_t n_chan, const double *uvw,
                        const double *freq, const double *image, size_t width,
                        size_t height, double dl, double dm, double l_shift,
                        double m_shift, const int64_t *vis_index, size_t n_sel,
                        int n_threads, double *out) {
  (void)n_rows;
  size_t n_src = 0;
  for (size_t p = 0; p < width * height; ++p)
    if (image[p] != 0.0) ++n_src;
  double *src = (double *)malloc(sizeof(double) * 4 * (n_src + 1));
  size_t k = 0;
  for (size_t y = 0; y < height; ++y)
    for (size_t x = 0; x < width; ++x) {
      const double v = image[x + y * width];
      if (v == 0.0) continue;
      double l, m;
      pixel_lm(x, y, width, height, dl, dm, l_shift, m_shift, &l, &m);
      src[4 * k + 0] = l;
      src[4 * k + 1] = m;
      src[4 * k + 2] = pixel_nm1(l, m);
      src[4 * k + 3] = v;
      ++k;
    }
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 64)
  for (size_t i = 0; i < n_sel; ++i) {
    const int64_t e = vis_index[i];
    const size_t r = e / n_chan, c = e % n_chan;
    const double inv_lambda = freq[c] / C_LIGHT;
    const double u = uvw[3 * r] * inv_lambda, v = uvw[3 * r + 1] * inv_lambda,
                 w = uvw[3 * r + 2] * inv_lambda;
    double re = 0.0, im = 0.0;
    for (size_t j = 0; j < n_src; ++j) {
      const double *b = src + 4 * j;
      double s, cc;
      sincos_turns(u * b[0] + v * b[1] + w * b[2], &s, &cc);
      re += b[3] * cc;
      im += b[3] * s;
    }
    out[2 * i] = re;
    out[2 * i + 1] = im;
  }
  free(src);
}

/* ------------------------------------------------------------------------ */
/* ES kernel                                                                  */
/* ------------------------------------------------------------------------ */

double oracle_es_kernel(double beta, double z) {
  if (!(fabs(z) < 1.0)) return 0.0;
  return exp(beta * (sqrt(1.0 - z * z) - 1.0));
}

/* Gauss-Legendre nodes on [0, 1] (Golub-Welsch via Newton on P_n). */
#define GL_N 256
static double gl_x[GL_N], gl_w[GL_N];
static int gl_ready = 0;
static void gl_init(void) {
  if (gl_ready) return;
  const int n = 2 * GL_N; /* nodes of P_n on [-1,1], keep the positive half */
  for (int i = 0; i < GL_N; ++i) {
    double x = cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = x;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      const double dp = n * (x * p1 - p0) / (x * x - 1.0);
      const double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-16) break;
    }
    double p0 = 1.0, p1 = x;
    for (int k = 2; k <= n; ++k) {
      const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    const double dp = n * (x * p1 - p0) / (x * x - 1.0);
    gl_x[i] = x;
    gl_w[i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  gl_ready = 1;
}

/* psihat(f) = (W/2) int_{-1}^{1} phi(z) cos(pi f W z) dz, f in cycles/cell. */
double oracle_es_fourier(double beta, int support, double f) {
  gl_init();
  double acc = 0.0;
  for (int i = 0; i < GL_N; ++i)
    acc += gl_w[i] * oracle_es_kernel(beta, gl_x[i]) *
           cos(M_PI * f * support * gl_x[i]);
  return support * acc; /* (W/2) * 2 * half-range integral */
}

/* ------------------------------------------------------------------------ */
/* Bucketing                                                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
  int64_t iu, iv, ip;
  float fu, fv, fw;
  int64_t key;
} Footprint;

/* The coordinate step, operation by operation as the GPU pass performs it. */
static void footprint(const OraclePlan *P, const double *scale_u,
                      const double *scale_v, const double *scale_w,
                      double inv_dw, const double *uvw_row, size_t c,
                      Footprint *f) {
  const double half = 0.5 * (double)P->support;
  const double U = uvw_row[0] * scale_u[c];
  const double V = uvw_row[1] * scale_v[c];
  const double iu0 = ceil(U - half);
  const double iv0 = ceil(V - half);
  f->fu = (float)(iu0 - U);
  f->fv = (float)(iv0 - V);
  int64_t iu = (int64_t)iu0 % P->nu;
  if (iu < 0) iu += P->nu;
  int64_t iv = (int64_t)iv0 % P->nv;
  if (iv < 0) iv += P->nv;
  f->iu = iu;
  f->iv = iv;
  if (P->n_planes > 1) {
    const double wl = uvw_row[2] * scale_w[c];
    const double Pw = (wl - P->w0) * inv_dw;
    double ip0 = ceil(Pw - half);
    const double ip_max = (double)(P->n_planes - P->support);
    if (ip0 < 0.0) ip0 = 0.0;
    if (ip0 > ip_max) ip0 = ip_max;
    f->ip = (int64_t)ip0;
    f->fw = (float)(ip0 - Pw);
  } else {
    f->ip = 0;
    f->fw = 0.0f;
  }
  const int64_t ntu = P->nu / P->tile;
  const int64_t tile = (iv / P->tile) * ntu + iu / P->tile;
  /* spill class: does the footprint reach the tile to the right / above */
  const int right = (iu % P->tile) > P->tile - P->support;
  const int up = (iv % P->tile) > P->tile - P->support;
  const int64_t cls = right ? (up ? 2 : 1) : (up ? 3 : 0);
  f->key = (tile * 4 + cls) * P->n_planes + f->ip;
}

static void channel_scales(const OraclePlan *P, size_t n_chan,
                           const double *freq, double *su, double *sv,
                           double *sw) {
  const double gu = P->dl * (double)P->nu;
  const double gv = P->dm * (double)P->nv;
  for (size_t c = 0; c < n_chan; ++c) {
    const double fl = freq[c] / C_LIGHT;
    su[c] = fl * gu;
    sv[c] = fl * gv;
    sw[c] = fl;
  }
}

int64_t oracle_bucket(const OraclePlan *P, size_t n_rows, size_t n_chan,
                      const double *uvw, const double *freq, const float *vis,
                      int skip_zero, uint32_t *perm, int64_t *key, int32_t *iu,
                      int32_t *iv, int32_t *ip, float *fu, float *fv,
                      float *fw, int64_t *offsets) {
  double *su = malloc(sizeof(double) * n_chan), *sv = malloc(sizeof(double) * n_chan),
         *sw = malloc(sizeof(double) * n_chan);
  channel_scales(P, n_chan, freq, su, sv, sw);
  const double inv_dw = P->n_planes > 1 ? 1.0 / P->dw : 0.0;
  const int64_t n_keys =
      (P->nu / P->tile) * (P->nv / P->tile) * 4 * P->n_planes;
  const size_t n_el = n_rows * n_chan;
  int64_t *ekey = malloc(sizeof(int64_t) * (n_el + 1));
  uint8_t *ecorner = malloc(n_el + 1);
  size_t corner_count[257] = {0};
  memset(offsets, 0, sizeof(int64_t) * (n_keys + 1));
  for (size_t r = 0; r < n_rows; ++r)
    for (size_t c = 0; c < n_chan; ++c) {
      const size_t e = r * n_chan + c;
      if (skip_zero && vis[2 * e] == 0.0f && vis[2 * e + 1] == 0.0f) {
        ekey[e] = -1;
        continue;
      }
      Footprint f;
      footprint(P, su, sv, sw, inv_dw, uvw + 3 * r, c, &f);
      ekey[e] = f.key;
      /* the footprint corner inside its tile, the order within a key */
      ecorner[e] = (uint8_t)((f.iv % P->tile) * P->tile + f.iu % P->tile);
      corner_count[ecorner[e] + 1]++;
      offsets[f.key + 1]++;
    }
  /* stable order by corner, then a stable counting sort by key over it: the
   * samples come out by (key, corner, element index) */
  for (int b = 0; b < 256; ++b) corner_count[b + 1] += corner_count[b];
  size_t *by_corner = malloc(sizeof(size_t) * (n_el + 1));
  for (size_t e = 0; e < n_el; ++e)
    if (ekey[e] >= 0) by_corner[corner_count[ecorner[e]]++] = e;
  const size_t n_kept = corner_count[255];
  for (int64_t k = 0; k < n_keys; ++k) offsets[k + 1] += offsets[k];
  int64_t *cursor = malloc(sizeof(int64_t) * (n_keys + 1));
  memcpy(cursor, offsets, sizeof(int64_t) * (n_keys + 1));
  for (size_t i = 0; i < n_kept; ++i) {
    const size_t e = by_corner[i];
    const int64_t s = cursor[ekey[e]]++;
    perm[s] = (uint32_t)e;
  }
  free(by_corner);
  free(ecorner);
  const int64_t n_out = offsets[n_keys];
  for (int64_t s = 0; s < n_out; ++s) {
    const size_t e = perm[s];
    Footprint f;
    footprint(P, su, sv, sw, inv_dw, uvw + 3 * (e / n_chan), e % n_chan, &f);
    key[s] = f.key;
    iu[s] = (int32_t)f.iu;
    iv[s] = (int32_t)f.iv;
    ip[s] = (int32_t)f.ip;
    fu[s] = f.fu;
    fv[s] = f.fv;
    fw[s] = f.fw;
  }
  free(cursor);
  free(ekey);
  free(su);
  free(sv);
  free(sw);
  return n_out;
}

/* ------------------------------------------------------------------------ */
/* FFT (complex double, radix 2/3/4/5 Stockham autosort)                      */
/* ------------------------------------------------------------------------ */

typedef struct {
  int n, nf;
  int f[40];
  double *tw; /* exp(-2 pi i j / n), j < n */
} FftPlan;

static int fft_plan(int n, FftPlan *p) {
  p->n = n;
  p->nf = 0;
  p->tw = NULL;
  int m = n;
  while (m % 4 == 0) { p->f[p->nf++] = 4; m /= 4; }
  while (m % 2 == 0) { p->f[p->nf++] = 2; m /= 2; }
  while (m % 3 == 0) { p->f[p->nf++] = 3; m /= 3; }
  while (m % 5 == 0) { p->f[p->nf++] = 5; m /= 5; }
  if (m != 1) return -1;
  p->tw = (double *)malloc(sizeof(double) * 2 * n);
  for (int j = 0; j < n; ++j) {
    const double a = -TWO_PI * (double)j / (double)n;
    p->tw[2 * j] = cos(a);
    p->tw[2 * j + 1] = sin(a);
  }
  return 0;
}

static void fft_free(FftPlan *p) {
  free(p->tw);
  p->tw = NULL;
}

/* One transform of length n (Stockham autosort); x and y are n complex doubles
 * (interleaved); the result ends up in x.  sign = -1 forward, +1 backward
 * (unnormalised). */
static void fft_run(const FftPlan *P, double *x, double *y, int sign) {
  const int n = P->n;
  int p = 1;
  double *a = x, *b = y;
  for (int s = 0; s < P->nf; ++s) {
    const int R = P->f[s];
    const int nR = n / R;
    const int step = n / (p * R);
    /* roots of unity of order R */
    double rr[5], ri[5];
    for (int q = 0; q < R; ++q) {
      rr[q] = P->tw[2 * (q * (n / R))];
      ri[q] = sign * -P->tw[2 * (q * (n / R)) + 1];
    }
    for (int i = 0; i < nR; ++i) {
      const int k = i % p;
      double ur[5], ui[5];
      for (int t = 0; t < R; ++t) {
        double re = a[2 * (i + t * nR)], im = a[2 * (i + t * nR) + 1];
        if (t > 0 && k > 0) {
          const int j = t * k * step;
          const double c = P->tw[2 * j], sn = sign * -P->tw[2 * j + 1];
          const double tr = re * c - im * sn;
          im = re * sn + im * c;
          re = tr;
        }
        ur[t] = re;
        ui[t] = im;
      }
      const int j = (i - k) * R + k;
      for (int q = 0; q < R; ++q) {
        double sr = 0.0, si = 0.0;
        for (int t = 0; t < R; ++t) {
          const int e = (t * q) % R;
          sr += ur[t] * rr[e] - ui[t] * ri[e];
          si += ur[t] * ri[e] + ui[t] * rr[e];
        }
        b[2 * (j + q * p)] = sr;
        b[2 * (j + q * p) + 1] = si;
      }
    }
    p *= R;
    double *t = a;
    a = b;
    b = t;
  }
  if (a != x) memcpy(x, a, sizeof(double) * 2 * n);
}

/* ------------------------------------------------------------------------ */
/* FP64 CPU w-gridder                                                         */
/* ------------------------------------------------------------------------ */

typedef struct {
  double re, im;  /* visibility times the shift phase (inversion) or the phase
                     factor itself (prediction) */
  double kx[16], ky[16], kw[16];
  int64_t iu, iv, ip;
  size_t elem;
} GridVis;

static int prepare_vis(const OraclePlan *P, size_t n_rows, size_t n_chan,
                       const double *uvw, const double *freq, const float *vis,
                       int skip_zero, GridVis **out, size_t *n_out) {
  const int W = (int)P->support;
  if (W > 16) return -1;
  double *su = malloc(sizeof(double) * n_chan), *sv = malloc(sizeof(double) * n_chan),
         *sw = malloc(sizeof(double) * n_chan);
  channel_scales(P, n_chan, freq, su, sv, sw);
  const double inv_dw = P->n_planes > 1 ? 1.0 / P->dw : 0.0;
  size_t n = 0;
  for (size_t e = 0; e < n_rows * n_chan; ++e)
    if (!skip_zero || vis[2 * e] != 0.0f || vis[2 * e + 1] != 0.0f) ++n;
  GridVis *g = malloc(sizeof(GridVis) * (n + 1));
  size_t k = 0;
  for (size_t r = 0; r < n_rows; ++r)
    for (size_t c = 0; c < n_chan; ++c) {
      const size_t e = r * n_chan + c;
      if (skip_zero && vis[2 * e] == 0.0f && vis[2 * e + 1] == 0.0f) continue;
      Footprint f;
      footprint(P, su, sv, sw, inv_dw, uvw + 3 * r, c, &f);
      GridVis *v = &g[k++];
      v->iu = f.iu;
      v->iv = f.iv;
      v->ip = f.ip;
      v->elem = e;
      /* kernel values from the FP64 coordinates (not the float fractions) */
      const double half = 0.5 * W;
      const double U = uvw[3 * r] * su[c], V = uvw[3 * r + 1] * sv[c];
      const double du = ceil(U - half) - U, dv = ceil(V - half) - V;
      for (int j = 0; j < W; ++j) {
        v->kx[j] = oracle_es_kernel(P->beta, (du + j) / half);
        v->ky[j] = oracle_es_kernel(P->beta, (dv + j) / half);
      }
      const double wl = uvw[3 * r + 2] * sw[c];
      if (P->n_planes > 1) {
        const double Pw = (wl - P->w0) * inv_dw;
        const double dw0 = (double)f.ip - Pw;
        for (int j = 0; j < W; ++j)
          v->kw[j] = oracle_es_kernel(P->beta, (dw0 + j) / half);
      } else {
        for (int j = 0; j < W; ++j) v->kw[j] = (j == 0) ? 1.0 : 0.0;
      }
      const double ul = uvw[3 * r] * sw[c], vl = uvw[3 * r + 1] * sw[c];
      double s, cc;
      sincos_turns(ul * P->l_shift + vl * P->m_shift + wl * P->nm1_center, &s,
                   &cc);
      if (vis) {
        /* V exp(-2 pi i theta) */
        const double re = vis[2 * e], im = vis[2 * e + 1];
        v->re = re * cc + im * s;
        v->im = im * cc - re * s;
      } else {
        v->re = cc;
        v->im = -s;
      }
    }
  *out = g;
  *n_out = n;
  free(su);
  free(sv);
  free(sw);
  return 0;
}

static int plane_count_w(const OraclePlan *P) {
  return P->n_planes > 1 ? (int)P->support : 1;
}

/* Grid correction 1 / (psihat_x psihat_y psihat_w) for every trimmed pixel. */
static void correction_table(const OraclePlan *P, const double *nu_w,
                             double *corr) {
  gl_init();
  const int64_t W = P->width, H = P->height;
  double *cx = malloc(sizeof(double) * W), *cy = malloc(sizeof(double) * H);
  for (int64_t x = 0; x < W; ++x)
    cx[x] = oracle_es_fourier(P->beta, (int)P->support,
                              (double)(W / 2 - x) / (double)P->nu);
  for (int64_t y = 0; y < H; ++y)
    cy[y] = oracle_es_fourier(P->beta, (int)P->support,
                              (double)(y - H / 2) / (double)P->nv);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < W * H; ++i) {
    double c = cx[i % W] * cy[i / W];
    if (P->n_planes > 1)
      c *= oracle_es_fourier(P->beta, (int)P->support, P->dw * nu_w[i]);
    corr[i] = 1.0 / c;
  }
  free(cx);
  free(cy);
}

/* Row stripes of the grid: samples whose footprint starts in stripe s write
 * rows [s * stripe, s * stripe + stripe + W - 1), so stripes two apart never
 * share a row and can be gridded by different threads. */
static int64_t stripe_rows(const OraclePlan *P) {
  return 64 > P->support ? 64 : P->support;
}
static int64_t stripe_count(const OraclePlan *P) {
  const int64_t n = P->nv / stripe_rows(P);
  return n > 0 ? n : 1;
}
static int64_t stripe_of(const OraclePlan *P, int64_t iv) {
  const int64_t s = iv / stripe_rows(P);
  return s < stripe_count(P) ? s : stripe_count(P) - 1;
}

/* grid all vis touching plane p into grid (nv x nu complex doubles).  sorder /
 * sstart list the samples of first plane q and stripe s (index
 * q * n_stripes + s) by footprint corner; every cell therefore receives its
 * samples in ascending (first plane, corner, sample) order. */
static void grid_plane(const OraclePlan *P, const GridVis *g, size_t n,
                       const size_t *sorder, const size_t *sstart, int p,
                       double *grid, int clear) {
  const int W = (int)P->support, nW = plane_count_w(P);
  const int64_t nu = P->nu, nv = P->nv;
  if (clear) memset(grid, 0, sizeof(double) * 2 * nu * nv);
  /* vis with ip in [p - nW + 1, p]; grouped by stripe parity for threads */
  const int64_t n_stripes = stripe_count(P);
  for (int color = 0; color < 3; ++color) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t s = 0; s < n_stripes; ++s) {
      int c = (int)(s & 1);
      if ((n_stripes & 1) && s == n_stripes - 1) c = 2;
      if (c != color) continue;
      for (int q = p - nW + 1; q <= p; ++q) {
        if (q < 0) continue;
        const size_t b = (size_t)q * (size_t)n_stripes + (size_t)s;
        for (size_t ii = sstart[b]; ii < sstart[b + 1]; ++ii) {
          const GridVis *v = &g[sorder[ii]];
          const double kwv = v->kw[p - q];
          for (int j = 0; j < W; ++j) {
            const int64_t row = (v->iv + j) % nv;
            const double wy = kwv * v->ky[j];
            double *gr = grid + 2 * row * nu;
            for (int i = 0; i < W; ++i) {
              const int64_t col = (v->iu + i) % nu;
              const double wt = wy * v->kx[i];
              gr[2 * col] += wt * v->re;
              gr[2 * col + 1] += wt * v->im;
            }
          }
        }
      }
    }
  }
  (void)n;
}

/* forward FFT of rows then of the cropped columns; writes the image-domain
 * values of the trimmed pixels into img (width*height complex, [x + y w]). */
static void fft_forward_crop(const OraclePlan *P, double *grid, double *img) {
  const int64_t nu = P->nu, nv = P->nv, W = P->width, H = P->height;
  FftPlan pu, pv;
  fft_plan((int)nu, &pu);
  fft_plan((int)nv, &pv);
#pragma omp parallel
  {
    double *tmp = malloc(sizeof(double) * 2 * (nu > nv ? nu : nv));
    double *col = malloc(sizeof(double) * 2 * nv);
#pragma omp for schedule(static)
    for (int64_t r = 0; r < nv; ++r) fft_run(&pu, grid + 2 * r * nu, tmp, -1);
#pragma omp for schedule(static)
    for (int64_t x = 0; x < W; ++x) {
      int64_t X = W / 2 - x;
      int64_t a = ((X % nu) + nu) % nu;
      for (int64_t b = 0; b < nv; ++b) {
        col[2 * b] = grid[2 * (b * nu + a)];
        col[2 * b + 1] = grid[2 * (b * nu + a) + 1];
      }
      fft_run(&pv, col, tmp, -1);
      for (int64_t y = 0; y < H; ++y) {
        int64_t Y = y - H / 2;
        int64_t bb = ((Y % nv) + nv) % nv;
        img[2 * (x + y * W)] = col[2 * bb];
        img[2 * (x + y * W) + 1] = col[2 * bb + 1];
      }
    }
    free(tmp);
    free(col);
  }
  fft_free(&pu);
  fft_free(&pv);
}

static void pixel_nu_table(const OraclePlan *P, double *nu_w) {
  for (int64_t y = 0; y < P->height; ++y)
    for (int64_t x = 0; x < P->width; ++x) {
      double l, m;
      pixel_lm(x, y, P->width, P->height, P->dl, P->dm, P->l_shift, P->m_shift,
               &l, &m);
      nu_w[x + y * P->width] = pixel_nm1(l, m) - P->nm1_center;
    }
}

static void sort_by_plane(const OraclePlan *P, const GridVis *g, size_t n,
                          size_t **order, size_t **pstart) {
  const int64_t np = P->n_planes;
  size_t *st = calloc(np + 2, sizeof(size_t));
  for (size_t i = 0; i < n; ++i) st[g[i].ip + 1]++;
  for (int64_t q = 0; q < np; ++q) st[q + 1] += st[q];
  size_t *cur = malloc(sizeof(size_t) * (np + 1));
  memcpy(cur, st, sizeof(size_t) * (np + 1));
  size_t *o = malloc(sizeof(size_t) * (n + 1));
  for (size_t i = 0; i < n; ++i) o[cur[g[i].ip]++] = i;
  free(cur);
  *order = o;
  *pstart = st;
}

typedef struct {
  int64_t corner; /* iv * nu + iu */
  size_t index;
} CornerKey;

static int corner_cmp(const void *a, const void *b) {
  const CornerKey *x = (const CornerKey *)a, *y = (const CornerKey *)b;
  if (x->corner != y->corner) return x->corner < y->corner ? -1 : 1;
  return x->index < y->index ? -1 : (x->index > y->index);
}

/* Counting sort of the samples by (first plane, stripe), each bucket ordered
 * by footprint corner (iv, iu) and then by sample index, so that a thread
 * walks its stripe's cells in address order: sorder lists the samples,
 * sstart[q * n_stripes + s] is where bucket (q, s) begins. */
static void sort_by_plane_stripe(const OraclePlan *P, const GridVis *g, size_t n,
                                 size_t **sorder, size_t **sstart) {
  const size_t ns = (size_t)stripe_count(P);
  const size_t nb = (size_t)P->n_planes * ns;
  size_t *st = calloc(nb + 2, sizeof(size_t));
  for (size_t i = 0; i < n; ++i)
    st[(size_t)g[i].ip * ns + (size_t)stripe_of(P, g[i].iv) + 1]++;
  for (size_t b = 0; b < nb; ++b) st[b + 1] += st[b];
  size_t *cur = malloc(sizeof(size_t) * (nb + 1));
  memcpy(cur, st, sizeof(size_t) * (nb + 1));
  CornerKey *k = malloc(sizeof(CornerKey) * (n + 1));
  for (size_t i = 0; i < n; ++i) {
    CornerKey *e = &k[cur[(size_t)g[i].ip * ns + (size_t)stripe_of(P, g[i].iv)]++];
    e->corner = g[i].iv * P->nu + g[i].iu;
    e->index = i;
  }
  free(cur);
#pragma omp parallel for schedule(dynamic, 16)
  for (size_t b = 0; b < nb; ++b)
    if (st[b + 1] - st[b] > 1) qsort(k + st[b], st[b + 1] - st[b], sizeof(CornerKey), corner_cmp);
  size_t *o = malloc(sizeof(size_t) * (n + 1));
  for (size_t i = 0; i < n; ++i) o[i] = k[i].index;
  free(k);
  *sorder = o;
  *sstart = st;
}

int oracle_wgrid_invert(const OraclePlan *P, size_t n_rows, size_t n_chan,
                        const double *uvw, const double *freq, const float *vis,
                        int n_threads, double *dirty) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
  FftPlan t1, t2;
  if (fft_plan((int)P->nu, &t1) || fft_plan((int)P->nv, &t2)) return -2;
  fft_free(&t1);
  fft_free(&t2);
  GridVis *g;
  size_t n;
  if (prepare_vis(P, n_rows, n_chan, uvw, freq, vis, 1, &g, &n)) return -1;
  size_t *order, *pstart;
  sort_by_plane_stripe(P, g, n, &order, &pstart);
  const int64_t W = P->width, H = P->height;
  double *grid = malloc(sizeof(double) * 2 * P->nu * P->nv);
  double *img = malloc(sizeof(double) * 2 * W * H);
  double *nu_w = malloc(sizeof(double) * W * H);
  pixel_nu_table(P, nu_w);
  memset(dirty, 0, sizeof(double) * W * H);
  for (int p = 0; p < P->n_planes; ++p) {
    grid_plane(P, g, n, order, pstart, p, grid, 1);
    fft_forward_crop(P, grid, img);
    const double wp = P->w0 + (double)p * P->dw;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < W * H; ++i) {
      double s, c;
      sincos_turns(wp * nu_w[i], &s, &c);
      /* Re(F exp(-2 pi i w_p nu)) */
      dirty[i] += img[2 * i] * c + img[2 * i + 1] * s;
    }
  }
  double *corr = malloc(sizeof(double) * W * H);
  correction_table(P, nu_w, corr);
  for (int64_t i = 0; i < W * H; ++i) dirty[i] *= corr[i];
  free(corr);
  free(grid);
  free(img);
  free(nu_w);
  free(order);
  free(pstart);
  free(g);
  return 0;
}

int oracle_wgrid_predict(const OraclePlan *P, size_t n_rows, size_t n_chan,
                         const double *uvw, const double *freq,
                         const double *image, int n_threads, double *vis_out) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
  FftPlan pu, pv;
  if (fft_plan((int)P->nu, &pu) || fft_plan((int)P->nv, &pv)) return -2;
  GridVis *g;
  size_t n;
  if (prepare_vis(P, n_rows, n_chan, uvw, freq, NULL, 0, &g, &n)) return -1;
  size_t *order, *pstart;
  sort_by_plane(P, g, n, &order, &pstart);
  const int64_t W = P->width, H = P->height, nu = P->nu, nv = P->nv;
  const int nW = plane_count_w(P);
  const int Ws = (int)P->support;
  double *grid = malloc(sizeof(double) * 2 * nu * nv);
  double *nu_w = malloc(sizeof(double) * W * H);
  double *corr = malloc(sizeof(double) * W * H);
  double *acc = calloc(2 * n + 2, sizeof(double));
  pixel_nu_table(P, nu_w);
  correction_table(P, nu_w, corr);
  for (int64_t i = 0; i < W * H; ++i) corr[i] *= image[i];
  for (int p = 0; p < P->n_planes; ++p) {
    const double wp = P->w0 + (double)p * P->dw;
    memset(grid, 0, sizeof(double) * 2 * nu * nv);
    /* scatter the screened image into the columns it occupies, then inverse
     * column FFTs over those columns and inverse row FFTs over every row. */
#pragma omp parallel
    {
      double *col = malloc(sizeof(double) * 2 * nv);
      double *tmp = malloc(sizeof(double) * 2 * (nu > nv ? nu : nv));
#pragma omp for schedule(static)
      for (int64_t x = 0; x < W; ++x) {
        memset(col, 0, sizeof(double) * 2 * nv);
        for (int64_t y = 0; y < H; ++y) {
          const int64_t i = x + y * W;
          double s, c;
          sincos_turns(wp * nu_w[i], &s, &c);
          const int64_t bb = (((y - H / 2) % nv) + nv) % nv;
          col[2 * bb] = corr[i] * c;
          col[2 * bb + 1] = corr[i] * s;
        }
        fft_run(&pv, col, tmp, +1);
        const int64_t a = (((W / 2 - x) % nu) + nu) % nu;
        for (int64_t b = 0; b < nv; ++b) {
          grid[2 * (b * nu + a)] = col[2 * b];
          grid[2 * (b * nu + a) + 1] = col[2 * b + 1];
        }
      }
#pragma omp for schedule(static)
      for (int64_t r = 0; r < nv; ++r) fft_run(&pu, grid + 2 * r * nu, tmp, +1);
      free(col);
      free(tmp);
    }
    for (int q = p - nW + 1; q <= p; ++q) {
      if (q < 0) continue;
#pragma omp parallel for schedule(static)
      for (size_t ii = pstart[q]; ii < pstart[q + 1]; ++ii) {
        const size_t k = order[ii];
        const GridVis *v = &g[k];
        const double kwv = v->kw[p - q];
        double sr = 0.0, si = 0.0;
        for (int j = 0; j < Ws; ++j) {
          const int64_t row = (v->iv + j) % nv;
          const double wy = kwv * v->ky[j];
          const double *gr = grid + 2 * row * nu;
          for (int i = 0; i < Ws; ++i) {
            const int64_t col = (v->iu + i) % nu;
            const double wt = wy * v->kx[i];
            sr += wt * gr[2 * col];
            si += wt * gr[2 * col + 1];
          }
        }
        acc[2 * k] += sr;
        acc[2 * k + 1] += si;
      }
    }
  }
  memset(vis_out, 0, sizeof(double) * 2 * n_rows * n_chan);
  for (size_t k = 0; k < n; ++k) {
    /* multiply by exp(+2 pi i theta) = conj(phase factor) */
    const double pr = g[k].re, pi = -g[k].im;
    const double ar = acc[2 * k], ai = acc[2 * k + 1];
    vis_out[2 * g[k].elem] = ar * pr - ai * pi;
    vis_out[2 * g[k].elem + 1] = ar * pi + ai * pr;
  }
  free(grid);
  free(nu_w);
  free(corr);
  free(acc);
  free(order);
  free(pstart);
  free(g);
  fft_free(&pu);
  fft_free(&pv);
  return 0;
}

/* Rows and columns of one plane pass that a timing run of `fraction` of a
 * pass transforms (at least one of each). */
static int64_t timed_count(int64_t total, double fraction) {
  int64_t k = (int64_t)ceil(fraction * (double)total);
  if (k < 1) k = 1;
  return k < total ? k : total;
}

double oracle_wgrid_time_parts(const OraclePlan *P, size_t n_rows,
                               size_t n_chan, const double *uvw,
                               const double *freq, const float *vis,
                               int n_threads, double plane_fraction,
                               double *plane_seconds) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
  const int64_t nu = P->nu, nv = P->nv, W = P->width, H = P->height;
  FftPlan pu, pv;
  if (fft_plan((int)nu, &pu) || fft_plan((int)nv, &pv)) return -1.0;
  const double t0 = omp_get_wtime();
  GridVis *g;
  size_t n;
  if (prepare_vis(P, n_rows, n_chan, uvw, freq, vis, 1, &g, &n)) return -1.0;
  size_t *order, *pstart;
  sort_by_plane_stripe(P, g, n, &order, &pstart);
  double *grid = calloc(2 * nu * nv, sizeof(double));
  /* spreading cost of every sample over all the planes it touches (the
   * per-plane clearing is charged to the plane part below) */
  for (int p = 0; p < P->n_planes; ++p)
    grid_plane(P, g, n, order, pstart, p, grid, 0);
  const double t1 = omp_get_wtime();
  double *nu_w = malloc(sizeof(double) * W * H);
  double *dirty = calloc(W * H, sizeof(double));
  pixel_nu_table(P, nu_w);
  const int64_t rows_t = timed_count(nv, plane_fraction);
  const int64_t cols_t = timed_count(W, plane_fraction);
  const double wp = P->w0;
  const double t2 = omp_get_wtime();
  /* `plane_fraction` of one inversion plane pass (fft_forward_crop plus the
   * screen): clear and transform rows_t rows, then cols_t cropped columns,
   * screened and accumulated into their pixels */
  memset(grid, 0, sizeof(double) * 2 * nu * rows_t);
#pragma omp parallel
  {
    double *tmp = malloc(sizeof(double) * 2 * (nu > nv ? nu : nv));
    double *col = malloc(sizeof(double) * 2 * nv);
#pragma omp for schedule(static)
    for (int64_t r = 0; r < rows_t; ++r) fft_run(&pu, grid + 2 * r * nu, tmp, -1);
#pragma omp for schedule(static)
    for (int64_t x = 0; x < cols_t; ++x) {
      const int64_t a = (((W / 2 - x) % nu) + nu) % nu;
      for (int64_t b = 0; b < nv; ++b) {
        col[2 * b] = grid[2 * (b * nu + a)];
        col[2 * b + 1] = grid[2 * (b * nu + a) + 1];
      }
      fft_run(&pv, col, tmp, -1);
      for (int64_t y = 0; y < H; ++y) {
        const int64_t bb = (((y - H / 2) % nv) + nv) % nv;
        const int64_t i = x + y * W;
        double sn, cs;
        sincos_turns(wp * nu_w[i], &sn, &cs);
        dirty[i] += col[2 * bb] * cs + col[2 * bb + 1] * sn;
      }
    }
    free(tmp);
    free(col);
  }
  const double t3 = omp_get_wtime();
  *plane_seconds = t3 - t2;
  free(grid);
  free(nu_w);
  free(dirty);
  free(order);
  free(pstart);
  free(g);
  fft_free(&pu);
  fft_free(&pv);
  return t1 - t0;
}

double oracle_wgrid_time_predict_parts(const OraclePlan *P, size_t n_rows,
                                       size_t n_chan, const double *uvw,
                                       const double *freq, const float *vis,
                                       int n_threads, double plane_fraction,
                                       double *plane_seconds) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
  const int64_t W = P->width, H = P->height, nu = P->nu, nv = P->nv;
  const int nW = plane_count_w(P), Ws = (int)P->support;
  FftPlan pu, pv;
  if (fft_plan((int)nu, &pu) || fft_plan((int)nv, &pv)) return -1.0;
  /* a plane in real (written) memory, so that the interpolation reads real
   * pages rather than the kernel's shared zero page */
  double *grid = malloc(sizeof(double) * 2 * nu * nv);
  memset(grid, 0, sizeof(double) * 2 * nu * nv);
  const double t0 = omp_get_wtime();
  GridVis *g;
  size_t n;
  /* the samples a masked prediction evaluates (vis != 0) */
  if (prepare_vis(P, n_rows, n_chan, uvw, freq, vis, 1, &g, &n)) return -1.0;
  size_t *order, *pstart;
  sort_by_plane(P, g, n, &order, &pstart);
  double *acc = calloc(2 * n + 2, sizeof(double));
  /* interpolation of every sample over all the planes it touches, as in
   * oracle_wgrid_predict (the plane transforms are charged below) */
  for (int p = 0; p < P->n_planes; ++p) {
    for (int q = p - nW + 1; q <= p; ++q) {
      if (q < 0) continue;
#pragma omp parallel for schedule(static)
      for (size_t ii = pstart[q]; ii < pstart[q + 1]; ++ii) {
        const size_t k = order[ii];
        const GridVis *v = &g[k];
        const double kwv = v->kw[p - q];
        double sr = 0.0, si = 0.0;
        for (int j = 0; j < Ws; ++j) {
          const int64_t row = (v->iv + j) % nv;
          const double wy = kwv * v->ky[j];
          const double *gr = grid + 2 * row * nu;
          for (int i = 0; i < Ws; ++i) {
            const int64_t col = (v->iu + i) % nu;
            const double wt = wy * v->kx[i];
            sr += wt * gr[2 * col];
            si += wt * gr[2 * col + 1];
          }
        }
        acc[2 * k] += sr;
        acc[2 * k + 1] += si;
      }
    }
  }
  const double t1 = omp_get_wtime();
  double *nu_w = malloc(sizeof(double) * W * H);
  double *corr = calloc(W * H, sizeof(double));
  pixel_nu_table(P, nu_w);
  memset(grid, 0, sizeof(double) * 2 * nu * nv);
  const double t2 = omp_get_wtime();
  /* `plane_fraction` of one prediction plane pass: the screened image into
   * cols_t of its columns with their inverse column FFTs, then rows_t inverse
   * row FFTs */
  const int64_t rows_t = timed_count(nv, plane_fraction);
  const int64_t cols_t = timed_count(W, plane_fraction);
  const double wp = P->w0;
#pragma omp parallel
  {
    double *col = malloc(sizeof(double) * 2 * nv);
    double *tmp = malloc(sizeof(double) * 2 * (nu > nv ? nu : nv));
#pragma omp for schedule(static)
    for (int64_t x = 0; x < cols_t; ++x) {
      memset(col, 0, sizeof(double) * 2 * nv);
      for (int64_t y = 0; y < H; ++y) {
        const int64_t i = x + y * W;
        double s, c;
        sincos_turns(wp * nu_w[i], &s, &c);
        const int64_t bb = (((y - H / 2) % nv) + nv) % nv;
        col[2 * bb] = corr[i] * c;
        col[2 * bb + 1] = corr[i] * s;
      }
      fft_run(&pv, col, tmp, +1);
      const int64_t a = (((W / 2 - x) % nu) + nu) % nu;
      for (int64_t b = 0; b < nv; ++b) {
        grid[2 * (b * nu + a)] = col[2 * b];
        grid[2 * (b * nu + a) + 1] = col[2 * b + 1];
      }
    }
#pragma omp for schedule(static)
    for (int64_t r = 0; r < rows_t; ++r) fft_run(&pu, grid + 2 * r * nu, tmp, +1);
    free(col);
    free(tmp);
  }
  const double t3 = omp_get_wtime();
  *plane_seconds = t3 - t2;
  free(grid);
  free(acc);
  free(nu_w);
  free(corr);
  free(order);
  free(pstart);
  free(g);
  fft_free(&pu);
  fft_free(&pv);
  return t1 - t0;
}

/* ------------------------------------------------------------------------ */
/* Gains and collapse                                                         */
/* ------------------------------------------------------------------------ */

typedef struct {
  float re, im;
} cf;
static inline cf cmul(cf a, cf b) {
  cf r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
  return r;
}
static inline cf cconj(cf a) {
  cf r = {a.re, -a.im};
  return r;
}
static inline cf cadd(cf a, cf b) {
  cf r = {a.re + b.re, a.im + b.im};
  return r;
}
static inline cf cscale(cf a, float s) {
  cf r = {a.re * s, a.im * s};
  return r;
}
static inline cf ld(const float *p, int i) {
  cf r = {p[2 * i], p[2 * i + 1]};
  return r;
}
static inline void st(float *p, int i, cf v) {
  p[2 * i] = v.re;
  p[2 * i + 1] = v.im;
}

/* 2x2 products on row-major [xx xy; yx yy] */
static void m_mul(const cf *a, const cf *b, cf *r) {
  r[0] = cadd(cmul(a[0], b[0]), cmul(a[1], b[2]));
  r[1] = cadd(cmul(a[0], b[1]), cmul(a[1], b[3]));
  r[2] = cadd(cmul(a[2], b[0]), cmul(a[3], b[2]));
  r[3] = cadd(cmul(a[2], b[1]), cmul(a[3], b[3]));
}
/* a^H b */
static void m_herm_mul(const cf *a, const cf *b, cf *r) {
  cf ah[4] = {cconj(a[0]), cconj(a[2]), cconj(a[1]), cconj(a[3])};
  m_mul(ah, b, r);
}
/* a b^H */
static void m_mul_herm(const cf *a, const cf *b, cf *r) {
  cf bh[4] = {cconj(b[0]), cconj(b[2]), cconj(b[1]), cconj(b[3])};
  m_mul(a, bh, r);
}

/* visibilitymodifier.h:378-401 */
void oracle_apply_conjugated_gain(int mode, float *vis, const float *g1p,
                                  const float *g2p) {
  cf g1[4], g2[4];
  for (int i = 0; i < 4; ++i) {
    g1[i] = ld(g1p, i);
    g2[i] = ld(g2p, i);
  }
  switch (mode) {
    case 0:
      st(vis, 0, cmul(cmul(cconj(g1[0]), ld(vis, 0)), g2[0]));
      break;
    case 1:
      st(vis, 0, cmul(cmul(cconj(g1[3]), ld(vis, 0)), g2[3]));
      break;
    case 2: {
      /* 0.5 * DoubleDot(g2, conj(g1)) */
      cf dd = {0.0f, 0.0f};
      for (int i = 0; i < 4; ++i) dd = cadd(dd, cmul(g2[i], cconj(g1[i])));
      st(vis, 0, cmul(ld(vis, 0), cscale(dd, 0.5f)));
      break;
    }
    case 3: {
      /* the second line reads the already-updated visibilities[0], exactly
       * as visibilitymodifier.h:393-396 does */
      cf v0 = cadd(cmul(cmul(cconj(g1[0]), ld(vis, 0)), g2[0]),
                   cmul(cmul(cconj(g1[2]), ld(vis, 1)), g2[2]));
      st(vis, 0, v0);
      cf v1 = cadd(cmul(cmul(cconj(g1[3]), ld(vis, 1)), g2[3]),
                   cmul(cmul(cconj(g1[1]), ld(vis, 0)), g2[1]));
      st(vis, 1, v1);
      break;
    }
    case 4: {
      cf v[4] = {ld(vis, 0), ld(vis, 1), ld(vis, 2), ld(vis, 3)}, t[4], r[4];
      m_herm_mul(g1, v, t);
      m_mul(t, g2, r);
      for (int i = 0; i < 4; ++i) st(vis, i, r[i]);
      break;
    }
  }
}

/* visibilitymodifier.h:345-369 (forward direction, for the KAT only) */
void oracle_apply_gain(int mode, float *vis, const float *g1p,
                       const float *g2p) {
  cf g1[4], g2[4];
  for (int i = 0; i < 4; ++i) {
    g1[i] = ld(g1p, i);
    g2[i] = ld(g2p, i);
  }
  switch (mode) {
    case 0:
      st(vis, 0, cmul(cmul(g1[0], ld(vis, 0)), cconj(g2[0])));
      break;
    case 1:
      st(vis, 0, cmul(cmul(g1[3], ld(vis, 0)), cconj(g2[3])));
      break;
    case 2: {
      cf dd = {0.0f, 0.0f};
      for (int i = 0; i < 4; ++i) dd = cadd(dd, cmul(g1[i], cconj(g2[i])));
      st(vis, 0, cmul(ld(vis, 0), cscale(dd, 0.5f)));
      break;
    }
    case 3: {
      cf v0 = cadd(cmul(cmul(g1[0], ld(vis, 0)), cconj(g2[0])),
                   cmul(cmul(g1[1], ld(vis, 1)), cconj(g2[1])));
      st(vis, 0, v0);
      cf v1 = cadd(cmul(cmul(g1[3], ld(vis, 1)), cconj(g2[3])),
                   cmul(cmul(g1[2], ld(vis, 0)), cconj(g2[2])));
      st(vis, 1, v1);
      break;
    }
    case 4: {
      cf v[4] = {ld(vis, 0), ld(vis, 1), ld(vis, 2), ld(vis, 3)}, t[4], r[4];
      m_mul(g1, v, t);
      m_mul_herm(t, g2, r);
      for (int i = 0; i < 4; ++i) st(vis, i, r[i]);
      break;
    }
  }
}

static int mode_npol(int mode) {
  switch (mode) {
    case 0: case 1: case 2: return 1;
    case 3: return 2;
    case 4: return 4;
  }
  return 0;
}

/* 4-pol collapse: linear-feed Stokes definitions (aocommon's
 * Polarization::ConvertFromLinear is absent; the 1/2 normalisation is the
 * standard one and is unpinned). */
static cf collapse4(const float *v, int pol) {
  cf xx = ld(v, 0), xy = ld(v, 1), yx = ld(v, 2), yy = ld(v, 3);
  switch (pol) {
    case 0: return cscale(cadd(xx, yy), 0.5f);
    case 1: { cf r = {0.5f * (xx.re - yy.re), 0.5f * (xx.im - yy.im)}; return r; }
    case 2: return cscale(cadd(xy, yx), 0.5f);
    case 3: {
      /* V = i (yx - xy) / 2 */
      cf d = {yx.re - xy.re, yx.im - xy.im};
      cf r = {-0.5f * d.im, 0.5f * d.re};
      return r;
    }
    case 4: return xx;
    case 5: return xy;
    case 6: return yx;
    default: return yy;
  }
}

/* Stokes parameter `pol` (or linear correlation 4-7) of value s as linear
 * correlations (XX, XY, YX, YY): the inverse of collapse4, i.e. XX = I + Q,
 * YY = I - Q, XY = U + iV, YX = U - iV.  This restates the 4-polarisation
 * branch of ExpandData (msgridderdata.h:63-68), whose converter
 * (aocommon::Polarization::ConvertToLinear) is absent from the reference tree:
 * the convention is the one of collapse4 above, unpinned. */
static void expand4(cf s, int pol, float *v) {
  cf z = {0.0f, 0.0f}, o[4] = {z, z, z, z};
  switch (pol) {
    case 0: o[0] = s; o[3] = s; break;
    case 1: { cf m = {-s.re, -s.im}; o[0] = s; o[3] = m; break; }
    case 2: o[1] = s; o[2] = s; break;
    case 3: { cf is = {-s.im, s.re}, mis = {s.im, -s.re}; o[1] = is; o[2] = mis; break; }
    case 4: o[0] = s; break;
    case 5: o[1] = s; break;
    case 6: o[2] = s; break;
    default: o[3] = s; break;
  }
  for (int i = 0; i < 4; ++i) st(v, i, o[i]);
}

int oracle_forward_gains(int mode, size_t n_pol, size_t n_rows, size_t n_chan,
                         const float *vis_in, const uint64_t *antenna_pairs,
                         const uint64_t *time_offsets, const float *solutions,
                         size_t nparms, size_t n_ant, int polarization, float *out) {
  if (mode_npol(mode) != (int)n_pol) return -1;
  if (nparms != 2 && nparms != 4) return -1;
  for (size_t r = 0; r < n_rows; ++r) {
    const uint64_t a1 = antenna_pairs[2 * r], a2 = antenna_pairs[2 * r + 1];
    const uint64_t t = time_offsets[r];
    for (size_t ch = 0; ch < n_chan; ++ch) {
      /* visibilitymodifier.cpp:205-227 indexing */
      const size_t off = (t * n_chan + ch) * n_ant * nparms;
      const float *s1 = solutions + 2 * (off + a1 * nparms);
      const float *s2 = solutions + 2 * (off + a2 * nparms);
      float g1[8] = {0}, g2[8] = {0};
      if (nparms == 2) {
        g1[0] = s1[0]; g1[1] = s1[1]; g1[6] = s1[2]; g1[7] = s1[3];
        g2[0] = s2[0]; g2[1] = s2[1]; g2[6] = s2[2]; g2[7] = s2[3];
      } else {
        memcpy(g1, s1, sizeof(float) * 8);
        memcpy(g2, s2, sizeof(float) * 8);
      }
      const cf sv = ld(vis_in + 2 * (r * n_chan + ch), 0);
      float v[8];
      if (n_pol == 1) {
        st(v, 0, sv);
      } else if (n_pol == 2) { /* ExpandData<2>, msgridderdata.h:58-62 */
        st(v, 0, sv);
        st(v, 1, sv);
      } else {
        expand4(sv, polarization, v);
      }
      oracle_apply_gain(mode, v, g1, g2); /* ApplyParmResponse -> ApplyGain */
      memcpy(out + 2 * ((r * n_chan + ch) * n_pol), v, sizeof(float) * 2 * n_pol);
    }
  }
  return 0;
}

int oracle_apply_gains(int mode, size_t n_pol, size_t n_rows, size_t n_chan,
                       const float *vis_in, const uint64_t *antenna_pairs,
                       const uint64_t *time_offsets, const float *solutions,
                       size_t nparms, size_t n_ant, int polarization,
                       float *out) {
  if (mode_npol(mode) != (int)n_pol) return -1;
  if (nparms != 2 && nparms != 4) return -1;
  for (size_t r = 0; r < n_rows; ++r) {
    const uint64_t a1 = antenna_pairs[2 * r], a2 = antenna_pairs[2 * r + 1];
    const uint64_t t = time_offsets[r];
    for (size_t ch = 0; ch < n_chan; ++ch) {
      /* msgridderdata.h / visibilitymodifier.h:549-551 indexing */
      const size_t off = (t * n_chan + ch) * n_ant * nparms;
      const float *s1 = solutions + 2 * (off + a1 * nparms);
      const float *s2 = solutions + 2 * (off + a2 * nparms);
      float g1[8] = {0}, g2[8] = {0};
      if (nparms == 2) {
        g1[0] = s1[0]; g1[1] = s1[1]; g1[6] = s1[2]; g1[7] = s1[3];
        g2[0] = s2[0]; g2[1] = s2[1]; g2[6] = s2[2]; g2[7] = s2[3];
      } else {
        memcpy(g1, s1, sizeof(float) * 8);
        memcpy(g2, s2, sizeof(float) * 8);
      }
      float v[8];
      memcpy(v, vis_in + 2 * ((r * n_chan + ch) * n_pol), sizeof(float) * 2 * n_pol);
      oracle_apply_conjugated_gain(mode, v, g1, g2);
      cf res;
      if (n_pol == 1) res = ld(v, 0);
      else if (n_pol == 2) res = cadd(ld(v, 0), ld(v, 1)); /* msgridderdata.h:41-45 */
      else res = collapse4(v, polarization);
      out[2 * (r * n_chan + ch)] = res.re;
      out[2 * (r * n_chan + ch) + 1] = res.im;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Imaging weights (structures/imageweights.{h,cpp}) and raw-row weighting    */
/* (gridding/msgridderdata.h:36-52, 760-886).                                 */
/* ------------------------------------------------------------------------ */

void oracle_weights_dims(size_t image_width, size_t image_height, double super_weight,
                         int64_t *width, int64_t *height) {
  int64_t w = (int64_t)round((double)image_width / super_weight);
  int64_t h = (int64_t)round((double)image_height / super_weight);
  if (w % 2 != 0) ++w;
  if (h % 2 != 0) ++h;
  *width = w;
  *height = h;
}

/* uvToXY + isWithinLimits (imageweights.h:74-96); -1 outside the grid. */
static int64_t weights_cell(double u, double v, int64_t W, int64_t H, double psx, double psy) {
  if (v < 0.0) {
    u = -u;
    v = -v;
  }
  const double fx = floor(u * (double)W * psx + (double)(W / 2));
  const double fy = floor(v * (double)H * psy);
  if (!(fx >= 0.0 && fx < (double)W && fy >= 0.0 && fy < (double)(H / 2))) return -1;
  return (int64_t)fx + (int64_t)fy * W;
}

/* xyToUV (imageweights.h:83-91). */
static void weights_uv(int64_t x, int64_t y, int64_t W, int64_t H, double psx, double psy,
                       double *u, double *v) {
  *u = (double)(x - W / 2) / ((double)W * psx);
  *v = (double)y / ((double)H * psy);
}

/* tukeyFrom0ToN (imageweights.h:114-116). */
static double weights_tukey(double x, double n) {
  return 0.5 * (1.0 + cos((M_PI / n) * (x - n)));
}

double oracle_weights_grid(double *grid, int64_t W, int64_t H, double psx, double psy,
                           int as_taper, size_t n_rows, size_t n_chan, size_t n_pol,
                           const double *uvw, const double *freq, const float *weights) {
  double total = 0.0;
  for (size_t r = 0; r < n_rows; ++r) {
    double um = uvw[3 * r], vm = uvw[3 * r + 1];
    if (vm < 0.0) {
      um = -um;
      vm = -vm;
    }
    for (size_t ch = 0; ch < n_chan; ++ch) {
      const double lambda = C_LIGHT / freq[ch];
      const double u = um / lambda, v = vm / lambda;
      for (size_t p = 0; p < n_pol; ++p) {
        float w = weights[(r * n_chan + ch) * n_pol + p];
        if (as_taper && w != 0.0f) w = 1.0f;
        const int64_t cell = weights_cell(u, v, W, H, psx, psy);
        if (cell >= 0) {
          grid[cell] += w;
          total += w;
        }
      }
    }
  }
  return total;
}

void oracle_weights_finish(double *grid, int64_t W, int64_t H, int mode, double robustness,
                           double total_sum) {
  const int64_t n = W * (H / 2);
  if (mode == 2) {
    double avg_w = 0.0;
    for (int64_t i = 0; i < n; ++i) avg_w += grid[i] * grid[i];
    avg_w /= total_sum;
    const double numerator_sqrt = 5.0 * exp((-M_LN10) * robustness);
    const double s_sq = numerator_sqrt * numerator_sqrt / avg_w;
    for (int64_t i = 0; i < n; ++i)
      if (grid[i] != 0.0) grid[i] = 1.0 / (1.0 + grid[i] * s_sq);
  } else if (mode == 1) {
    for (int64_t i = 0; i < n; ++i) grid[i] = grid[i] != 0.0 ? 1.0 / grid[i] : 0.0;
  } else {
    for (int64_t i = 0; i < n; ++i)
      if (grid[i] != 0.0) grid[i] = 1.0;
  }
}

/* windowMean (imageweights.cpp:353-388). */
static double weights_window_mean(const double *grid, int64_t W, int64_t Hh, int64_t x,
                                  int64_t y, int64_t window) {
  const int64_t d = window / 2;
  const int64_t x1 = x <= d ? 0 : x - d, y1 = y <= d ? 0 : y - d;
  const int64_t x2 = x + d >= W ? W : x + d, y2 = y + d >= Hh ? Hh : y + d;
  int64_t count = 0;
  double sum = 0.0;
  for (int64_t yi = y1; yi < y2; ++yi)
    for (int64_t xi = x1; xi < x2; ++xi) {
      const double w = grid[yi * W + xi];
      if (w != 0.0) {
        ++count;
        sum += w;
      }
    }
  return sum / (double)count;
}

void oracle_weights_taper(double *grid, int64_t W, int64_t H, double psx, double psy, int kind,
                          double a, double b) {
  const int64_t Hh = H / 2, n = W * Hh;
  if (kind == 7) { /* RankFilter (imageweights.cpp:310-326) */
    double *src = (double *)malloc(sizeof(double) * (size_t)n);
    memcpy(src, grid, sizeof(double) * (size_t)n);
    for (int64_t y = 0; y < Hh; ++y)
      for (int64_t x = 0; x < W; ++x) {
        const double w = src[y * W + x];
        if (w != 0.0) {
          const double mean = weights_window_mean(src, W, Hh, x, y, (int64_t)b);
          if (w > mean * a) grid[y * W + x] = mean * a;
        }
      }
    free(src);
    return;
  }
  double m2s2 = 0.0, max_u = 0.0, max_v = 0.0;
  if (kind == 6) { /* SetGaussianTaper (imageweights.cpp:328-351) */
    const double half_power_uv = 1.0 / (a * 2.0 * M_PI);
    const long double sigma_to_hp = 2.0L * sqrtl(2.0L * logl(2.0L));
    m2s2 = half_power_uv * sigma_to_hp;
    m2s2 *= -2.0 * m2s2;
  }
  weights_uv(W, Hh, W, H, psx, psy, &max_u, &max_v);
  for (int64_t y = 0; y < Hh; ++y)
    for (int64_t x = 0; x < W; ++x) {
      double *g = grid + y * W + x;
      double u, v;
      weights_uv(x, y, W, H, psx, psy, &u, &v);
      const double d2 = u * u + v * v;
      switch (kind) {
        case 0: /* SetMinUVRange (:149-165) */
          if (d2 < a * a) *g = 0.0;
          break;
        case 1: /* SetMaxUVRange (:167-183) */
          if (d2 > a * a) *g = 0.0;
          break;
        case 2: /* SetTukeyTaper (:185-208): a transition, b max uv */
          if (d2 > b * b)
            *g = 0.0;
          else if (d2 > (b - a) * (b - a))
            *g *= weights_tukey(b - sqrt(d2), a);
          break;
        case 3: /* SetTukeyInnerTaper (:210-233): a transition, b min uv */
          if (d2 < b * b)
            *g = 0.0;
          else if (d2 < (b + a) * (b + a))
            *g *= weights_tukey(sqrt(d2) - b, a);
          break;
        case 4: /* SetEdgeTaper (:235-252) */
          if (max_u - fabs(u) < a || max_v - fabs(v) < a) *g = 0.0;
          break;
        case 5: { /* SetEdgeTukeyTaper (:254-282): a transition, b edge */
          const double ud = max_u - fabs(u), vd = max_v - fabs(v), total = a + b;
          if (ud < b || vd < b) {
            *g = 0.0;
          } else if (ud < total || vd < total) {
            double ru = ud - b, rv = vd - b;
            if (ru > a) ru = a;
            if (rv > a) rv = a;
            *g *= weights_tukey(ru, a) * weights_tukey(rv, a);
          }
          break;
        }
        case 6:
          if (*g != 0.0) *g = *g * exp(d2 / m2s2);
          break;
        default:
          break;
      }
    }
}

void oracle_weights_mirror(const double *grid, int64_t W, int64_t H, double *image) {
  for (int64_t y = 0; y < H / 2; ++y)
    for (int64_t x = 0; x < W; ++x) {
      image[(H / 2 - 1 - y) * W + (W - x - 1)] = grid[y * W + x];
      image[(H / 2 + y) * W + x] = grid[y * W + x];
    }
}

void oracle_weights_sample(const double *grid, int64_t W, int64_t H, double psx, double psy,
                           size_t n, const double *u, const double *v, double *out) {
  for (size_t i = 0; i < n; ++i) {
    const int64_t cell = weights_cell(u[i], v[i], W, H, psx, psy);
    out[i] = cell >= 0 ? grid[cell] : 0.0;
  }
}

/* AverageCorrection::Add for the modes with a matrix sum (every mode but
 * TRACE, averagecorrection.h:36-50): the Kronecker products a = G1 (x) G2 and
 * b = G2 (x) G1 of the 2 x 2 gains (row-major, complex64 pairs) in double, and
 * 0.5 w (a^H a + b^H b) added to sum, the 4 x 4 complex matrix row-major as
 * 32 doubles (re, im).  Element ((i, k), (j, l)) of G1 (x) G2 is
 * G1[i][j] G2[k][l], at row 2 i + k and column 2 j + l. */
void oracle_correction_matrix_add(const float *g1, const float *g2, double w, double *sum) {
  double a[32], b[32];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j)
      for (int k = 0; k < 2; ++k)
        for (int l = 0; l < 2; ++l) {
          const int at = 2 * ((2 * i + k) * 4 + 2 * j + l);
          const double x1 = g1[2 * (2 * i + j)], y1 = g1[2 * (2 * i + j) + 1];
          const double x2 = g2[2 * (2 * k + l)], y2 = g2[2 * (2 * k + l) + 1];
          a[at] = x1 * x2 - y1 * y2;
          a[at + 1] = x1 * y2 + y1 * x2;
          const double u1 = g2[2 * (2 * i + j)], v1 = g2[2 * (2 * i + j) + 1];
          const double u2 = g1[2 * (2 * k + l)], v2 = g1[2 * (2 * k + l) + 1];
          b[at] = u1 * u2 - v1 * v2;
          b[at + 1] = u1 * v2 + v1 * u2;
        }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double re = 0.0, im = 0.0;
      for (int q = 0; q < 4; ++q) {
        /* conj(m[q][r]) m[q][c] for m = a and b */
        const double *ar = a + 2 * (q * 4 + r), *ac = a + 2 * (q * 4 + c);
        const double *br = b + 2 * (q * 4 + r), *bc = b + 2 * (q * 4 + c);
        re += ar[0] * ac[0] + ar[1] * ac[1] + br[0] * bc[0] + br[1] * bc[1];
        im += ar[0] * ac[1] - ar[1] * ac[0] + br[0] * bc[1] - br[1] * bc[0];
      }
      sum[2 * (r * 4 + c)] += 0.5 * w * re;
      sum[2 * (r * 4 + c) + 1] += 0.5 * w * im;
    }
}

/* With a gain table (sol != NULL): ApplyConjugatedParmResponse between the
 * weighting and ApplyWeights (msgridderdata.h:888-927,
 * visibilitymodifier.h:538-594), and the AverageCorrection sum
 * (averagecorrection.h:36-50): for TRACE the scalar into corr[0], for the other
 * modes the matrix into corr[1..32] (oracle_correction_matrix_add). */
static void prepare_rows_impl(const double *grid, int64_t W, int64_t H, double psx, double psy,
                              int psf_mode, double psf_dl, double psf_dm, int subtract_model,
                              int visibility_weighting, int polarization, size_t n_pol,
                              size_t n_rows, size_t n_chan, const double *uvw, const double *freq,
                              const float *vis, const float *weights, const float *model,
                              const uint8_t *selected, float *vis_out, float *weights_out,
                              float *imaging_out, double *sums, int mode,
                              const uint64_t *antenna_pairs, const uint64_t *time_offsets,
                              const float *solutions, size_t nparms, size_t n_ant, double *corr) {
  float *row = (float *)malloc(sizeof(float) * 2 * n_chan * n_pol);
  float *wrow = (float *)malloc(sizeof(float) * n_chan * n_pol);
  float *scratch_iw = (float *)malloc(sizeof(float) * n_chan);
  for (size_t r = 0; r < n_rows; ++r) {
    const double *ruvw = uvw + 3 * r;
    const size_t base = r * n_chan * n_pol;
    memcpy(wrow, weights + base, sizeof(float) * n_chan * n_pol);
    if (psf_mode != 0) { /* msgridderdata.h:826-843 */
      for (size_t i = 0; i < n_chan * n_pol; ++i) {
        row[2 * i] = 1.0f;
        row[2 * i + 1] = 0.0f;
      }
      if (psf_dl != 0.0 || psf_dm != 0.0) {
        const double dn = sqrt(1.0 - psf_dl * psf_dl - psf_dm * psf_dm) - 1.0;
        const double shift = 2.0 * M_PI * (ruvw[0] * psf_dl + ruvw[1] * psf_dm + ruvw[2] * dn);
        for (size_t ch = 0; ch < n_chan; ++ch) { /* RotateVisibilities, :929-941 */
          const double rad = shift / (C_LIGHT / freq[ch]);
          const cf ph = {(float)cos(rad), (float)sin(rad)};
          for (size_t p = 0; p < n_pol; ++p) {
            float *c = row + 2 * (ch * n_pol + p);
            st(c, 0, cmul(ld(c, 0), ph));
          }
        }
      }
    } else {
      memcpy(row, vis + 2 * base, sizeof(float) * 2 * n_chan * n_pol);
    }
    if (subtract_model) /* :845-852 */
      for (size_t i = 0; i < 2 * n_chan * n_pol; ++i) row[i] -= model[2 * base + i];
    for (size_t ch = 0; ch < n_chan; ++ch) /* :857-862 */
      if (selected && !selected[r * n_chan + ch])
        for (size_t p = 0; p < n_pol; ++p) wrow[ch * n_pol + p] = 0.0f;
    for (size_t i = 0; i < n_chan * n_pol; ++i) { /* :864-878 */
      if (visibility_weighting == 1)
        wrow[i] *= wrow[i];
      else if (visibility_weighting == 2 && wrow[i] != 0.0f)
        wrow[i] = 1.0f;
    }
    for (size_t ch = 0; ch < n_chan; ++ch) { /* :880-885 */
      const double lambda = C_LIGHT / freq[ch];
      double w;
      oracle_weights_sample(grid, W, H, psx, psy, 1, (const double[]){ruvw[0] / lambda},
                            (const double[]){ruvw[1] / lambda}, &w);
      scratch_iw[ch] = (float)w;
    }
    if (solutions) /* ApplyCorrections, visibilitymodifier.h:538-594 */
      for (size_t ch = 0; ch < n_chan; ++ch) {
        const size_t off = (time_offsets[r] * n_chan + ch) * n_ant * nparms;
        const float *s1 = solutions + 2 * (off + antenna_pairs[2 * r] * nparms);
        const float *s2 = solutions + 2 * (off + antenna_pairs[2 * r + 1] * nparms);
        float g1[8] = {0}, g2[8] = {0};
        if (nparms == 2) {
          g1[0] = s1[0]; g1[1] = s1[1]; g1[6] = s1[2]; g1[7] = s1[3];
          g2[0] = s2[0]; g2[1] = s2[1]; g2[6] = s2[2]; g2[7] = s2[3];
        } else {
          memcpy(g1, s1, sizeof(float) * 8);
          memcpy(g2, s2, sizeof(float) * 8);
        }
        oracle_apply_conjugated_gain(mode, row + 2 * ch * n_pol, g1, g2);
        if (mode == 2) { /* AverageCorrection::Add, scalar (kTrace) */
          const cf a = cmul(ld(g2, 0), cconj(ld(g1, 0))), b = cmul(ld(g2, 3), cconj(ld(g1, 3)));
          const cf g = {0.5f * (a.re + b.re), 0.5f * (a.im + b.im)};
          const float norm = g.re * g.re + g.im * g.im;
          corr[0] += norm * (wrow[ch * n_pol] * scratch_iw[ch]);
        } else { /* the matrix form of the other modes */
          oracle_correction_matrix_add(g1, g2, (double)(wrow[ch * n_pol] * scratch_iw[ch]),
                                       corr + 1);
        }
      }
    for (size_t ch = 0; ch < n_chan; ++ch) /* ApplyWeights, :760-789 */
      for (size_t p = 0; p < n_pol; ++p) {
        const size_t i = ch * n_pol + p;
        const float cum = wrow[i] * scratch_iw[ch];
        const int has = cum != 0.0f;
        if (p == 0) {
          sums[0] += wrow[i] * (float)has;
          if ((double)cum > sums[1]) sums[1] = (double)cum;
          sums[3] += has;
        }
        sums[2] += cum;
        wrow[i] = cum;
        row[2 * i] *= cum;
        row[2 * i + 1] *= cum;
      }
    for (size_t ch = 0; ch < n_chan; ++ch) { /* CollapseData, :36-52 */
      const float *c = row + 2 * ch * n_pol;
      cf out;
      if (n_pol == 1)
        out = ld(c, 0);
      else if (n_pol == 2)
        out = cadd(ld(c, 0), ld(c, 1));
      else
        out = collapse4(c, polarization);
      st(vis_out + 2 * (r * n_chan + ch), 0, out);
      if (imaging_out) imaging_out[r * n_chan + ch] = scratch_iw[ch];
    }
    if (weights_out) memcpy(weights_out + base, wrow, sizeof(float) * n_chan * n_pol);
  }
  free(row);
  free(wrow);
  free(scratch_iw);
}

void oracle_prepare_rows(const double *grid, int64_t W, int64_t H, double psx, double psy,
                         int psf_mode, double psf_dl, double psf_dm, int subtract_model,
                         int visibility_weighting, int polarization, size_t n_pol,
                         size_t n_rows, size_t n_chan, const double *uvw, const double *freq,
                         const float *vis, const float *weights, const float *model,
                         const uint8_t *selected, float *vis_out, float *weights_out,
                         float *imaging_out, double *sums) {
  prepare_rows_impl(grid, W, H, psx, psy, psf_mode, psf_dl, psf_dm, subtract_model,
                    visibility_weighting, polarization, n_pol, n_rows, n_chan, uvw, freq, vis,
                    weights, model, selected, vis_out, weights_out, imaging_out, sums, 0, NULL,
                    NULL, NULL, 2, 0, NULL);
}

void oracle_prepare_rows_corrected(const double *grid, int64_t W, int64_t H, double psx,
                                   double psy, int psf_mode, double psf_dl, double psf_dm,
                                   int subtract_model, int visibility_weighting, int polarization,
                                   size_t n_pol, size_t n_rows, size_t n_chan, const double *uvw,
                                   const double *freq, const float *vis, const float *weights,
                                   const float *model, const uint8_t *selected, float *vis_out,
                                   float *weights_out, float *imaging_out, double *sums, int mode,
                                   const uint64_t *antenna_pairs, const uint64_t *time_offsets,
                                   const float *solutions, size_t nparms, size_t n_ant,
                                   double *correction_sum) {
  prepare_rows_impl(grid, W, H, psx, psy, psf_mode, psf_dl, psf_dm, subtract_model,
                    visibility_weighting, polarization, n_pol, n_rows, n_chan, uvw, freq, vis,
                    weights, model, selected, vis_out, weights_out, imaging_out, sums, mode,
                    antenna_pairs, time_offsets, solutions, nparms, n_ant, correction_sum);
}
