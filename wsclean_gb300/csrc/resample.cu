// Image resampling around the gridder boundary, on the device.
//
// WGriddingMSGridder::FinishInversion and StartPredict
// (wgridder/wgriddingmsgridder.cpp:273-340) change the image between the
// padded image size and the (smaller) inversion size chosen by the small
// inversion (gridding/msgridder.cpp:42-75, math/calculatefftsize.h) with
// schaapcommon's FFT resampler, and trim / untrim it around the centre.  The
// resampler restated here is the published FFT method: the real input's
// half spectrum (r2c), the rows [0, b_h / 2) and the last b_h / 2 rows of its
// first b_w / 2 + 1 columns (b = the smaller of the two sizes) copied into an
// otherwise zero half spectrum of the output size, the inverse (c2r) and a
// factor 1 / (in_w * in_h).  Non-finite input pixels (the NaN border of
// RealImage) count as zero.
//
// The transforms are batched mixed-radix Stockham passes (radices 2, 3, 4, 5,
// 7, 8 unrolled, other factors up to 64 generic), one launch per pass, over
// rows or columns of a complex work image in HBM.  Twiddles and the radix
// constants are computed on the host in double and stored as float.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "wgpu_internal.h"

namespace wgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxRadix = 64;

unsigned blocks_for(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

struct Stage {
  int radix;
  int64_t p;       // product of the radices of the earlier passes
  int64_t tw_off;  // twiddles exp(-2 pi i q k / (p R)), q in [1, R), k in [0, p)
  int64_t rc_off;  // radix constants exp(-2 pi i m / R), m in [0, R)
};

std::vector<int> factorize(int64_t n) {
  std::vector<int> f;
  while (n % 8 == 0) {
    f.push_back(8);
    n /= 8;
  }
  while (n % 4 == 0) {
    f.push_back(4);
    n /= 4;
  }
  for (int r : {2, 3, 5, 7}) {
    while (n % r == 0) {
      f.push_back(r);
      n /= r;
    }
  }
  for (int r = 11; n > 1 && r <= kMaxRadix; r += 2) {
    while (n % r == 0) {
      f.push_back(r);
      n /= r;
    }
  }
  if (n != 1) f.clear();  // a prime factor above kMaxRadix
  return f;
}

// Stages of a length-n transform, their twiddles appended to tw.
std::vector<Stage> plan_1d(int64_t n, std::vector<float2> &tw) {
  std::vector<Stage> st;
  if (n == 1) return st;
  const std::vector<int> f = factorize(n);
  if (f.empty())
    throw Error(WGPU_ERR_INVALID, "resampling size " + std::to_string(n) +
                                      " has a prime factor above 64");
  int64_t p = 1;
  for (int r : f) {
    Stage s;
    s.radix = r;
    s.p = p;
    s.tw_off = (int64_t)tw.size();
    for (int q = 1; q < r; ++q)
      for (int64_t k = 0; k < p; ++k) {
        const double a = -2.0 * M_PI * (double)q * (double)k / (double)(p * r);
        tw.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
      }
    s.rc_off = (int64_t)tw.size();
    for (int m = 0; m < r; ++m) {
      const double a = -2.0 * M_PI * (double)m / (double)r;
      tw.push_back(make_float2((float)std::cos(a), (float)std::sin(a)));
    }
    st.push_back(s);
    p *= r;
  }
  return st;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// One Stockham pass (Bainville's formulation): butterfly i in [0, n / R) reads
// x[i + q n / R], q in [0, R), multiplies by the twiddles of k = i mod p,
// transforms over q and writes y[(i - k) R + k + q p].  Sequence b of the
// batch starts at b * bstride; its elements are estride apart.
template <int R>
__device__ __forceinline__ void stage_body(const float2 *x, float2 *y, int64_t n, int64_t i,
                                           int64_t b, int64_t bstride, int64_t estride,
                                           int64_t p, const float2 *tw, const float2 *rc,
                                           int inverse, int radix) {
  constexpr int RM = R > 0 ? R : kMaxRadix;
  const int r = R > 0 ? R : radix;
  const int64_t nq = n / r;
  const int64_t k = i % p;
  const int64_t j = (i - k) * r + k;
  const float2 *xb = x + b * bstride;
  float2 *yb = y + b * bstride;
  float2 u[RM];
#pragma unroll
  for (int q = 0; q < RM; ++q) {
    if (q >= r) break;
    float2 v = xb[(i + q * nq) * estride];
    if (q > 0 && k > 0) {
      float2 w = tw[(q - 1) * p + k];
      if (inverse) w = cconj(w);
      v = cmul(v, w);
    }
    u[q] = v;
  }
#pragma unroll
  for (int o = 0; o < RM; ++o) {
    if (o >= r) break;
    float2 acc = u[0];
    for (int q = 1; q < r; ++q) {
      float2 w = rc[(q * o) % r];
      if (inverse) w = cconj(w);
      const float2 t = cmul(u[q], w);
      acc.x += t.x;
      acc.y += t.y;
    }
    yb[(j + o * p) * estride] = acc;
  }
}

template <int R>
__global__ void fft_stage_kernel(const float2 *x, float2 *y, int64_t n, int64_t batch,
                                 int64_t bstride, int64_t estride, int batch_fastest, int64_t p,
                                 const float2 *tw, const float2 *rc, int inverse, int radix) {
  const int r = R > 0 ? R : radix;
  const int64_t nq = n / r;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq * batch) return;
  int64_t i, b;
  if (batch_fastest) {
    b = t % batch;
    i = t / batch;
  } else {
    i = t % nq;
    b = t / nq;
  }
  stage_body<R>(x, y, n, i, b, bstride, estride, p, tw, rc, inverse, radix);
}

// Row transforms of power-of-two length n in [512, 8192] whose radices are
// 8, 4 and 2, in shared memory: one block of n / 16 threads per row loads the
// row once, runs every pass in place (each thread holds its 16 values in
// registers between the barriers of a pass) and writes the row once.  The
// butterflies i = threadIdx.x + b * blockDim.x, b < 16 / R, cover [0, n / R)
// exactly.
struct RowStages {
  int n_st;
  int radix[16];
  int p[16];
  int tw_off[16];
  int rc_off[16];
};

template <int R>
__device__ __forceinline__ void smem_pass(float2 *buf, int n, int p, const float2 *tw,
                                          const float2 *rc, int inverse) {
  constexpr int PER = 16 / R;
  const int nq = n / R;
  float2 out[16];
  int jj[PER];
#pragma unroll
  for (int b = 0; b < PER; ++b) {
    const int i = threadIdx.x + b * blockDim.x;
    const int k = i & (p - 1);
    jj[b] = (i - k) * R + k;
    float2 u[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      float2 v = buf[i + q * nq];
      if (q > 0 && k > 0) {
        float2 w = tw[(q - 1) * p + k];
        if (inverse) w = cconj(w);
        v = cmul(v, w);
      }
      u[q] = v;
    }
#pragma unroll
    for (int o = 0; o < R; ++o) {
      float2 acc = u[0];
#pragma unroll
      for (int q = 1; q < R; ++q) {
        float2 w = rc[(q * o) % R];
        if (inverse) w = cconj(w);
        const float2 t = cmul(u[q], w);
        acc.x += t.x;
        acc.y += t.y;
      }
      out[b * R + o] = acc;
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < PER; ++b)
#pragma unroll
    for (int o = 0; o < R; ++o) buf[jj[b] + o * p] = out[b * R + o];
  __syncthreads();
}

__global__ void __launch_bounds__(512, 2) fft_rows_smem_kernel(float2 *data, int n, int64_t stride,
                                                             RowStages st, const float2 *tw,
                                                             int inverse) {
  extern __shared__ float2 buf[];
  float2 *row = data + (int64_t)blockIdx.x * stride;
  for (int e = threadIdx.x; e < n; e += blockDim.x) buf[e] = row[e];
  __syncthreads();
  for (int s = 0; s < st.n_st; ++s) {
    const float2 *t = tw + st.tw_off[s], *rc = tw + st.rc_off[s];
    if (st.radix[s] == 8)
      smem_pass<8>(buf, n, st.p[s], t, rc, inverse);
    else if (st.radix[s] == 4)
      smem_pass<4>(buf, n, st.p[s], t, rc, inverse);
    else
      smem_pass<2>(buf, n, st.p[s], t, rc, inverse);
  }
  for (int e = threadIdx.x; e < n; e += blockDim.x) row[e] = buf[e];
}

bool rows_in_smem(const std::vector<Stage> &st, int64_t n) {
  if (n < 512 || n > 8192 || (n & (n - 1)) != 0 || st.size() > 16) return false;
  for (const Stage &g : st)
    if (g.radix != 8 && g.radix != 4 && g.radix != 2) return false;
  return true;
}

// Real image (row-major, w x h) -> complex work image, non-finite pixels 0.
__global__ void load_real_kernel(const float *in, int64_t n, float2 *a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float v = in[i];
  a[i] = make_float2(isfinite(v) ? v : 0.0f, 0.0f);
}

// The output half spectrum: rows [0, bh/2) and the last bh/2 rows of
// columns [0, bw/2] from the input spectrum, zero elsewhere; the columns
// above out_w / 2 are the conjugates of their mirror columns (the real
// output's Hermitian extension, applied after the inverse along y).
__global__ void copy_spectrum_kernel(const float2 *a, int64_t in_w, int64_t in_h, float2 *b,
                                     int64_t out_w, int64_t out_h) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t half = out_w / 2 + 1;
  if (i >= half * out_h) return;
  const int64_t ky = i / half, kx = i - ky * half;
  const int64_t bw = in_w < out_w ? in_w : out_w, bh = in_h < out_h ? in_h : out_h;
  float2 v = make_float2(0.0f, 0.0f);
  if (kx <= bw / 2) {
    if (ky < bh / 2)
      v = a[ky * in_w + kx];
    else if (ky >= out_h - bh / 2)
      v = a[(in_h - (out_h - ky)) * in_w + kx];
  }
  b[ky * out_w + kx] = v;
}

__global__ void hermitian_rows_kernel(float2 *b, int64_t out_w, int64_t out_h) {
  const int64_t half = out_w / 2 + 1, upper = out_w - half;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= upper * out_h) return;
  const int64_t y = i / upper, kx = half + (i - y * upper);
  b[y * out_w + kx] = cconj(b[y * out_w + (out_w - kx)]);
}

__global__ void store_real_kernel(const float2 *b, int64_t n, float scale, float *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = b[i].x * scale;
}

// Runs the passes of one batched transform, ping-ponging between *cur and
// *alt (on return *cur holds the result).
void run_fft(const std::vector<Stage> &st, float2 **cur, float2 **alt, int64_t n, int64_t batch,
             int64_t bstride, int64_t estride, bool batch_fastest, const float2 *d_tw,
             bool inverse, cudaStream_t s) {
  if (!batch_fastest && estride == 1 && rows_in_smem(st, n)) {
    RowStages rs{};
    rs.n_st = (int)st.size();
    for (size_t k = 0; k < st.size(); ++k) {
      rs.radix[k] = st[k].radix;
      rs.p[k] = (int)st[k].p;
      rs.tw_off[k] = (int)st[k].tw_off;
      rs.rc_off[k] = (int)st[k].rc_off;
    }
    const size_t smem = sizeof(float2) * (size_t)n;
    ensure_dynamic_smem((const void *)fft_rows_smem_kernel, smem);
    fft_rows_smem_kernel<<<(unsigned)batch, (unsigned)(n / 16), smem, s>>>(
        *cur, (int)n, bstride, rs, d_tw, inverse ? 1 : 0);
    check_launch("fft_rows_smem_kernel");
    return;  // transformed in place
  }
  for (const Stage &g : st) {
    const int64_t threads = n / g.radix * batch;
    const float2 *tw = d_tw + g.tw_off, *rc = d_tw + g.rc_off;
    const int bf = batch_fastest ? 1 : 0, inv = inverse ? 1 : 0;
#define WGPU_STAGE(RR)                                                                      \
  fft_stage_kernel<RR><<<blocks_for(threads), kThreads, 0, s>>>(                           \
      *cur, *alt, n, batch, bstride, estride, bf, g.p, tw, rc, inv, g.radix)
    switch (g.radix) {
      case 2: WGPU_STAGE(2); break;
      case 3: WGPU_STAGE(3); break;
      case 4: WGPU_STAGE(4); break;
      case 5: WGPU_STAGE(5); break;
      case 7: WGPU_STAGE(7); break;
      case 8: WGPU_STAGE(8); break;
      default: WGPU_STAGE(0); break;
    }
#undef WGPU_STAGE
    check_launch("fft_stage_kernel");
    std::swap(*cur, *alt);
  }
}

// Image::Trim / Untrim: the centred (out_w x out_h) window of a larger image
// starts at ((in_w - out_w) / 2, (in_h - out_h) / 2).
__global__ void trim_kernel(const float *in, int64_t in_w, int64_t in_h, float *out,
                            int64_t out_w, int64_t out_h) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= out_w * out_h) return;
  const int64_t y = i / out_w, x = i - y * out_w;
  out[i] = in[(x + (in_w - out_w) / 2) + (y + (in_h - out_h) / 2) * in_w];
}

__global__ void untrim_kernel(const float *in, int64_t in_w, int64_t in_h, float *out,
                              int64_t out_w, int64_t out_h) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= out_w * out_h) return;
  const int64_t y = i / out_w, x = i - y * out_w;
  const int64_t xs = x - (out_w - in_w) / 2, ys = y - (out_h - in_h) / 2;
  out[i] = (xs >= 0 && xs < in_w && ys >= 0 && ys < in_h) ? in[xs + ys * in_w] : 0.0f;
}

}  // namespace

void launch_trim(const float *in, int64_t in_w, int64_t in_h, float *out, int64_t out_w,
                 int64_t out_h, cudaStream_t s) {
  if (out_w > in_w || out_h > in_h) throw Error(WGPU_ERR_INVALID, "trim size above image size");
  trim_kernel<<<blocks_for(out_w * out_h), kThreads, 0, s>>>(in, in_w, in_h, out, out_w, out_h);
  check_launch("trim_kernel");
}

void launch_untrim(const float *in, int64_t in_w, int64_t in_h, float *out, int64_t out_w,
                   int64_t out_h, cudaStream_t s) {
  if (in_w > out_w || in_h > out_h) throw Error(WGPU_ERR_INVALID, "trim size above image size");
  untrim_kernel<<<blocks_for(out_w * out_h), kThreads, 0, s>>>(in, in_w, in_h, out, out_w,
                                                                out_h);
  check_launch("untrim_kernel");
}

size_t resample_work_bytes(int64_t in_w, int64_t in_h, int64_t out_w, int64_t out_h) {
  const int64_t cells = std::max(in_w * in_h, out_w * out_h);
  // two complex work images and the twiddles of four transforms
  const int64_t tw = 4 * (std::max(std::max(in_w, in_h), std::max(out_w, out_h)) * 2 + 64 * 8);
  return sizeof(float2) * (size_t)(2 * cells + tw) + 256;
}

void resample_device(const float *in, int64_t in_w, int64_t in_h, float *out, int64_t out_w,
                     int64_t out_h, void *work, cudaStream_t s) {
  if (in_w <= 0 || in_h <= 0 || out_w <= 0 || out_h <= 0)
    throw Error(WGPU_ERR_INVALID, "resampling sizes must be positive");
  std::vector<float2> tw;
  const std::vector<Stage> fx = plan_1d(in_w, tw), fy = plan_1d(in_h, tw);
  const std::vector<Stage> iy = plan_1d(out_h, tw), ix = plan_1d(out_w, tw);
  const int64_t cells = std::max(in_w * in_h, out_w * out_h);
  float2 *buf0 = (float2 *)work, *buf1 = buf0 + cells;
  float2 *d_tw = buf1 + cells;
  if ((int64_t)tw.size() > 4 * (std::max(std::max(in_w, in_h), std::max(out_w, out_h)) * 2 + 64 * 8))
    throw Error(WGPU_ERR_INVALID, "resampling twiddle table overflow");
  if (!tw.empty())
    WGPU_CUDA(cudaMemcpyAsync(d_tw, tw.data(), sizeof(float2) * tw.size(),
                              cudaMemcpyHostToDevice, s));
  float2 *cur = buf0, *alt = buf1;
  const int64_t n_in = in_w * in_h, n_out = out_w * out_h;
  load_real_kernel<<<blocks_for(n_in), kThreads, 0, s>>>(in, n_in, cur);
  check_launch("load_real_kernel");
  // r2c: rows (the full complex transform of real rows), then the columns
  // [0, in_w / 2] along y
  run_fft(fx, &cur, &alt, in_w, in_h, in_w, 1, false, d_tw, false, s);
  run_fft(fy, &cur, &alt, in_h, in_w / 2 + 1, 1, in_w, true, d_tw, false, s);
  copy_spectrum_kernel<<<blocks_for((out_w / 2 + 1) * out_h), kThreads, 0, s>>>(
      cur, in_w, in_h, alt, out_w, out_h);
  check_launch("copy_spectrum_kernel");
  std::swap(cur, alt);
  // c2r: columns [0, out_w / 2] along y, the rows' Hermitian extension, rows
  run_fft(iy, &cur, &alt, out_h, out_w / 2 + 1, 1, out_w, true, d_tw, true, s);
  if (out_w / 2 + 1 < out_w) {
    hermitian_rows_kernel<<<blocks_for((out_w - out_w / 2 - 1) * out_h), kThreads, 0, s>>>(
        cur, out_w, out_h);
    check_launch("hermitian_rows_kernel");
  }
  run_fft(ix, &cur, &alt, out_w, out_h, out_w, 1, false, d_tw, true, s);
  const float scale = (float)(1.0 / ((double)in_w * (double)in_h));
  store_real_kernel<<<blocks_for(n_out), kThreads, 0, s>>>(cur, n_out, scale, out);
  check_launch("store_real_kernel");
}

}  // namespace wgpu

// ---- C ABI ------------------------------------------------------------------

namespace {

template <typename F>
int resample_guarded(F &&fn) {
  try {
    wgpu::clear_failure();
    fn();
    return WGPU_OK;
  } catch (const wgpu::Error &e) {
    return wgpu::report_failure(e.status, e.what());
  } catch (const std::bad_alloc &) {
    return wgpu::report_failure(WGPU_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception &e) {
    return wgpu::report_failure(WGPU_ERR_INVALID, e.what());
  }
}

// hasLowPrimeFactors (math/calculatefftsize.h:8-20).
bool low_prime_factors(size_t n) {
  while (n > 7) {
    if (n % 2 == 0)
      n /= 2;
    else if (n % 3 == 0)
      n /= 3;
    else if (n % 5 == 0)
      n /= 5;
    else if (n % 7 == 0)
      n /= 7;
    else
      return false;
  }
  return true;
}

bool sizes_ok(size_t a, size_t b, size_t c, size_t d) {
  const size_t lim = (size_t)1 << 16;
  return a && b && c && d && a <= lim && b <= lim && c <= lim && d <= lim;
}

}  // namespace

extern "C" {

int wgpu_calculate_fft_size(size_t size, double pixel_scale, double beam_size,
                            size_t *minimal_size, size_t *optimal_size) {
  if (!minimal_size || !optimal_size) return wgpu::report_failure(WGPU_ERR_INVALID, "null output");
  if (!(pixel_scale > 0) || !(beam_size > 0))
    return wgpu::report_failure(WGPU_ERR_INVALID, "pixel scale and beam size must be > 0");
  // math/calculatefftsize.h:24-35
  const double total = (double)size * pixel_scale;
  const double m = std::ceil(total * 2 / beam_size);
  if (!(m >= 0 && m < 1e15)) return wgpu::report_failure(WGPU_ERR_INVALID, "size out of range");
  size_t opt = (size_t)m;
  *minimal_size = opt;
  if (opt % 4 != 0) opt += 4 - (opt % 4);
  while (!low_prime_factors(opt) && opt < size) opt += 4;
  if (opt > size) opt = size;
  *optimal_size = opt;
  wgpu::clear_failure();
  return WGPU_OK;
}

int wgpu_small_inversion_size(size_t width, size_t height, double pixel_size_x,
                              double pixel_size_y, double beam_size, size_t *inversion_width,
                              size_t *inversion_height, double *inversion_pixel_x,
                              double *inversion_pixel_y) {
  if (!inversion_width || !inversion_height || !inversion_pixel_x || !inversion_pixel_y)
    return wgpu::report_failure(WGPU_ERR_INVALID, "null output");
  size_t min_w, opt_w, min_h, opt_h;
  int st = wgpu_calculate_fft_size(width, pixel_size_x, beam_size, &min_w, &opt_w);
  if (st != WGPU_OK) return st;
  st = wgpu_calculate_fft_size(height, pixel_size_y, beam_size, &min_h, &opt_h);
  if (st != WGPU_OK) return st;
  // gridding/msgridder.cpp:42-75
  *inversion_width = width;
  *inversion_height = height;
  *inversion_pixel_x = pixel_size_x;
  *inversion_pixel_y = pixel_size_y;
  if (opt_w < width || opt_h < height) {
    const size_t nw = std::max(std::min(opt_w, width), (size_t)32);
    const size_t nh = std::max(std::min(opt_h, height), (size_t)32);
    *inversion_pixel_x = ((double)width * pixel_size_x) / (double)nw;
    *inversion_pixel_y = ((double)height * pixel_size_y) / (double)nh;
    *inversion_width = nw;
    *inversion_height = nh;
  }
  return WGPU_OK;
}

int wgpu_actual_trimmed_size(size_t inversion_width, size_t inversion_height,
                             double image_padding, size_t *trimmed_width,
                             size_t *trimmed_height) {
  if (!trimmed_width || !trimmed_height || !(image_padding > 0))
    return wgpu::report_failure(WGPU_ERR_INVALID, "invalid argument");
  // wgridder/wgriddingmsgridder.cpp:243-260
  size_t tw = (size_t)std::ceil((double)inversion_width / image_padding);
  size_t th = (size_t)std::ceil((double)inversion_height / image_padding);
  if (tw % 4 != 0) tw += 4 - (tw % 4);
  if (th % 4 != 0) th += 4 - (th % 4);
  *trimmed_width = std::min(tw, inversion_width);
  *trimmed_height = std::min(th, inversion_height);
  wgpu::clear_failure();
  return WGPU_OK;
}

int wgpu_resample_device(const float *d_in, size_t in_w, size_t in_h, float *d_out,
                         size_t out_w, size_t out_h, void *stream) {
  if (!d_in || !d_out) return wgpu::report_failure(WGPU_ERR_INVALID, "null argument");
  if (!sizes_ok(in_w, in_h, out_w, out_h))
    return wgpu::report_failure(WGPU_ERR_INVALID, "resampling sizes must be 1 to 65536");
  return resample_guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    void *work = nullptr;
    WGPU_CUDA(cudaMalloc(&work, wgpu::resample_work_bytes((int64_t)in_w, (int64_t)in_h,
                                                          (int64_t)out_w, (int64_t)out_h)));
    try {
      wgpu::resample_device(d_in, (int64_t)in_w, (int64_t)in_h, d_out, (int64_t)out_w,
                            (int64_t)out_h, work, s);
      WGPU_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
      cudaStreamSynchronize(s);
      cudaFree(work);
      throw;
    }
    WGPU_CUDA(cudaFree(work));
  });
}

int wgpu_resample(const float *in, size_t in_w, size_t in_h, float *out, size_t out_w,
                  size_t out_h) {
  if (!in || !out) return wgpu::report_failure(WGPU_ERR_INVALID, "null argument");
  if (!sizes_ok(in_w, in_h, out_w, out_h))
    return wgpu::report_failure(WGPU_ERR_INVALID, "resampling sizes must be 1 to 65536");
  int n_dev = 0;
  if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev == 0) {
    cudaGetLastError();
    return wgpu::report_failure(WGPU_ERR_CUDA, "no CUDA device");
  }
  float *d_in = nullptr, *d_out = nullptr;
  const int st = resample_guarded([&] {
    WGPU_CUDA(cudaMalloc(&d_in, sizeof(float) * in_w * in_h));
    WGPU_CUDA(cudaMalloc(&d_out, sizeof(float) * out_w * out_h));
    WGPU_CUDA(cudaMemcpy(d_in, in, sizeof(float) * in_w * in_h, cudaMemcpyHostToDevice));
  });
  int rs = st;
  if (st == WGPU_OK) rs = wgpu_resample_device(d_in, in_w, in_h, d_out, out_w, out_h, nullptr);
  if (rs == WGPU_OK)
    rs = resample_guarded([&] {
      WGPU_CUDA(cudaMemcpy(out, d_out, sizeof(float) * out_w * out_h, cudaMemcpyDeviceToHost));
    });
  if (d_in) cudaFree(d_in);
  if (d_out) cudaFree(d_out);
  return rs;
}

}  // extern "C"
