// oracle/dft_cuda.cu -- TEST INFRASTRUCTURE ONLY.
//
// FP64 direct Fourier transform on the GPU: the CUDA twin of oracle_dft_invert
// and oracle_dft_predict (wgpu_oracle.c).  It exists to measure the product's
// error over EVERY visibility of workloads far too large for the CPU oracle
// (hundreds of millions of samples against thousands of pixels).  Nothing in
// the product links, loads or calls it; tests/ and bench.py's accuracy leg use
// it as the checker, and a test pins it to the CPU oracle.
//
// Conventions restated from the reference's exact transform, as in the CPU
// oracle: phase t = (u l + v m + w (n - 1)) nu / c in turns with u, v, w in
// metres (gridding/directmsgridder.cpp:166-176), I(l, m) = sum Re(V e^{-2 pi i t})
// (:92-132), l = (width/2 - x) dl + l_shift, m = (y - height/2) dm + m_shift
// (:56-89, :113-124), n - 1 := 0 beyond the horizon (:205-229).
//
// Arithmetic.  Everything is FP64 (the samples are converted once from
// complex64).  For linearly spaced channels nu_c = nu_0 + c dnu the phase is
// t_c = t_0 + c d with t_0 = T nu_0 / c_light and d = T dnu / c_light, so
//   sum_c V_c e^{-2 pi i t_c} = e^{-2 pi i t_0} sum_c V_c z^c,  z = e^{-2 pi i d},
// which is evaluated by Horner's rule: two FP64 sincospi per (row, pixel) and
// one complex multiply-add per sample.  Both arguments are reduced modulo one
// turn in FP64 before sincospi.  Channels that are not linearly spaced (to
// 1e-12 relative) take one sincospi per sample instead.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr double kC = 299792458.0;
constexpr int kThreads = 128;
constexpr int kRowTile = 8;     // rows staged per round (inversion)
constexpr int kChanBlock = 16;  // channels per thread (prediction)

thread_local std::string g_error;

#define OC_CHECK(x)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess) {                                                         \
      g_error = std::string(#x) + ": " + cudaGetErrorString(e_);                     \
      return 1;                                                                      \
    }                                                                                \
  } while (0)

// A caller pointer that may be host or device memory: device memory is used in
// place, host memory is copied to a temporary device buffer.
struct DevView {
  const void *ptr = nullptr;
  void *owned = nullptr;
  ~DevView() {
    if (owned) cudaFree(owned);
  }
  int bind(const void *p, size_t bytes, cudaStream_t s) {
    if (p == nullptr) return 0;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess &&
        (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)) {
      ptr = p;
      return 0;
    }
    cudaGetLastError();
    OC_CHECK(cudaMalloc(&owned, bytes ? bytes : 1));
    OC_CHECK(cudaMemcpyAsync(owned, p, bytes, cudaMemcpyHostToDevice, s));
    ptr = owned;
    return 0;
  }
};

template <typename T>
struct DevArray {
  T *ptr = nullptr;
  ~DevArray() {
    if (ptr) cudaFree(ptr);
  }
  int alloc(size_t n) {
    OC_CHECK(cudaMalloc(&ptr, sizeof(T) * (n ? n : 1)));
    return 0;
  }
};

// Frequencies nu_c = nu_0 + c dnu to 1e-12 relative?
bool linear_channels(const double *freq, size_t n_chan, double *nu0, double *dnu) {
  *nu0 = freq[0];
  *dnu = n_chan > 1 ? (freq[n_chan - 1] - freq[0]) / (double)(n_chan - 1) : 0.0;
  double scale = 0.0;
  for (size_t c = 0; c < n_chan; ++c) scale = std::fmax(scale, std::fabs(freq[c]));
  for (size_t c = 0; c < n_chan; ++c)
    if (std::fabs(freq[c] - (*nu0 + (double)c * *dnu)) > 1e-12 * scale) return false;
  return true;
}

// l, m, n - 1 of trimmed pixel p = x + y width (the CPU oracle's pixel_lm and
// pixel_nm1).
void pixel_lmn(int64_t p, int64_t width, int64_t height, double dl, double dm, double l_shift,
               double m_shift, double *out) {
  const int64_t x = p % width, y = p / width;
  const double l = (double)(width / 2 - x) * dl + l_shift;
  const double m = (double)(y - height / 2) * dm + m_shift;
  const double r2 = l * l + m * m;
  out[0] = l;
  out[1] = m;
  out[2] = r2 >= 1.0 ? 0.0 : -r2 / (std::sqrt(1.0 - r2) + 1.0);
}

// Per row: one past the last channel with a non-zero sample (0: empty row).
__global__ void row_extent_kernel(const float2 *__restrict__ vis, int64_t n_rows, int n_chan,
                                  int *__restrict__ nc) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  int last = 0;
  for (int c = 0; c < n_chan; ++c) {
    const float2 v = vis[r * n_chan + c];
    if (v.x != 0.0f || v.y != 0.0f) last = c + 1;
  }
  nc[r] = last;
}

__device__ __forceinline__ double frac_turns(double t) { return t - rint(t); }

// Inversion: block (x, y) = (128 pixels, a contiguous range of rows).  Rows
// are staged kRowTile at a time (u, v, w and the samples as FP64), every thread
// evaluates its pixel against each staged row.  partial[y][pixel].
__global__ void __launch_bounds__(kThreads)
    dft_invert_kernel(const double *__restrict__ uvw, const float2 *__restrict__ vis,
                      const int *__restrict__ nc_row, int64_t n_rows, int n_chan,
                      int64_t rows_per_block, const double *__restrict__ freq, double nu0_c,
                      double dnu_c, int linear, const double *__restrict__ lmn, int n_pix,
                      double *__restrict__ partial) {
  extern __shared__ double2 s_vis[];  // [kRowTile][n_chan]
  __shared__ double s_uvw[kRowTile][3];
  __shared__ int s_nc[kRowTile];
  const int pix = blockIdx.x * kThreads + threadIdx.x;
  const bool active = pix < n_pix;
  double l = 0.0, m = 0.0, n = 0.0;
  if (active) {
    l = lmn[3 * pix];
    m = lmn[3 * pix + 1];
    n = lmn[3 * pix + 2];
  }
  const int64_t r_begin = (int64_t)blockIdx.y * rows_per_block;
  const int64_t r_end = r_begin + rows_per_block < n_rows ? r_begin + rows_per_block : n_rows;
  double acc = 0.0;
  for (int64_t r0 = r_begin; r0 < r_end; r0 += kRowTile) {
    __syncthreads();
    const int nr = (int)(r_end - r0 < kRowTile ? r_end - r0 : kRowTile);
    for (int i = threadIdx.x; i < kRowTile * n_chan; i += kThreads) {
      const int k = i / n_chan, c = i - k * n_chan;
      double2 v = make_double2(0.0, 0.0);
      if (k < nr) {
        const float2 f = vis[(r0 + k) * n_chan + c];
        v = make_double2((double)f.x, (double)f.y);
      }
      s_vis[i] = v;
    }
    if (threadIdx.x < kRowTile) {
      const int k = threadIdx.x;
      s_nc[k] = k < nr ? nc_row[r0 + k] : 0;
      for (int a = 0; a < 3; ++a) s_uvw[k][a] = k < nr ? uvw[3 * (r0 + k) + a] : 0.0;
    }
    __syncthreads();
    if (!active) continue;
    for (int k = 0; k < nr; ++k) {
      const int nc = s_nc[k];
      if (nc == 0) continue;
      const double T = fma(s_uvw[k][0], l, fma(s_uvw[k][1], m, s_uvw[k][2] * n));
      const double2 *v = s_vis + k * n_chan;
      if (linear) {
        double s0, c0, sd, cd;
        sincospi(2.0 * frac_turns(T * nu0_c), &s0, &c0);
        sincospi(2.0 * frac_turns(T * dnu_c), &sd, &cd);
        // Horner: h = sum_c V_c z^c, z = (cd, -sd)
        double hr = v[nc - 1].x, hi = v[nc - 1].y;
        for (int c = nc - 2; c >= 0; --c) {
          const double tr = fma(hr, cd, fma(hi, sd, v[c].x));
          const double ti = fma(hi, cd, fma(-hr, sd, v[c].y));
          hr = tr;
          hi = ti;
        }
        // Re(e^{-2 pi i t_0} h)
        acc += fma(c0, hr, s0 * hi);
      } else {
        for (int c = 0; c < nc; ++c) {
          double s, co;
          sincospi(2.0 * frac_turns(T * (freq[c] / kC)), &s, &co);
          acc += fma(v[c].x, co, v[c].y * s);
        }
      }
    }
  }
  if (active) partial[(size_t)blockIdx.y * n_pix + pix] = acc;
}

struct Source {
  double l, m, n, flux;
};

// Prediction: one thread per (row, block of kChanBlock channels), all sources
// staged in shared memory tiles.  V_c = sum_s S_s e^{+2 pi i t_c}.  Writes the
// values (ref, optional) and per-block partial sums of |pred - ref|^2 and
// |ref|^2 over the selected samples (mask != 0, or all when mask is null).
__global__ void __launch_bounds__(kThreads)
    dft_predict_kernel(const double *__restrict__ uvw, int64_t n_rows, int n_chan,
                       const double *__restrict__ freq, double dnu_c, int linear,
                       const Source *__restrict__ src, int n_src,
                       const uint8_t *__restrict__ mask, const float2 *__restrict__ pred,
                       double2 *__restrict__ ref_out, double *__restrict__ partial) {
  __shared__ Source s_src[kThreads];
  __shared__ double s_red[2][kThreads / 32];
  const int n_cb = (n_chan + kChanBlock - 1) / kChanBlock;
  const int64_t t = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool active = t < n_rows * n_cb;
  const int64_t row = active ? t / n_cb : 0;
  const int c0 = active ? (int)(t - row * n_cb) * kChanBlock : 0;
  const int kn = active ? (n_chan - c0 < kChanBlock ? n_chan - c0 : kChanBlock) : 0;
  const double u = active ? uvw[3 * row] : 0.0, v = active ? uvw[3 * row + 1] : 0.0,
               w = active ? uvw[3 * row + 2] : 0.0;
  const double nu0_c = active ? freq[c0] / kC : 0.0;
  double ar[kChanBlock], ai[kChanBlock];
#pragma unroll
  for (int k = 0; k < kChanBlock; ++k) ar[k] = ai[k] = 0.0;
  for (int s0 = 0; s0 < n_src; s0 += kThreads) {
    __syncthreads();
    if (s0 + threadIdx.x < n_src) s_src[threadIdx.x] = src[s0 + threadIdx.x];
    __syncthreads();
    const int ns = n_src - s0 < kThreads ? n_src - s0 : kThreads;
    if (!active) continue;
    for (int j = 0; j < ns; ++j) {
      const Source q = s_src[j];
      const double T = fma(u, q.l, fma(v, q.m, w * q.n));
      if (linear) {
        double sp, cp, sz, cz;
        sincospi(2.0 * frac_turns(T * nu0_c), &sp, &cp);
        sincospi(2.0 * frac_turns(T * dnu_c), &sz, &cz);
        double pr = q.flux * cp, pi = q.flux * sp;
#pragma unroll
        for (int k = 0; k < kChanBlock; ++k) {
          ar[k] += pr;
          ai[k] += pi;
          const double tr = fma(pr, cz, -pi * sz);
          pi = fma(pi, cz, pr * sz);
          pr = tr;
        }
      } else {
#pragma unroll
        for (int k = 0; k < kChanBlock; ++k) {
          if (k < kn) {
            double s, co;
            sincospi(2.0 * frac_turns(T * (freq[c0 + k] / kC)), &s, &co);
            ar[k] = fma(q.flux, co, ar[k]);
            ai[k] = fma(q.flux, s, ai[k]);
          }
        }
      }
    }
  }
  double e2 = 0.0, r2 = 0.0;
#pragma unroll
  for (int k = 0; k < kChanBlock; ++k) {
    if (k < kn) {
      const int64_t e = row * n_chan + c0 + k;
      if (ref_out) ref_out[e] = make_double2(ar[k], ai[k]);
      if (mask == nullptr || mask[e] != 0) {
        r2 += ar[k] * ar[k] + ai[k] * ai[k];
        if (pred) {
          const float2 p = pred[e];
          const double dr = (double)p.x - ar[k], di = (double)p.y - ai[k];
          e2 += dr * dr + di * di;
        }
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    r2 += __shfl_xor_sync(0xffffffffu, r2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_red[0][threadIdx.x >> 5] = e2;
    s_red[1][threadIdx.x >> 5] = r2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < kThreads / 32; ++i) {
      a += s_red[0][i];
      b += s_red[1][i];
    }
    partial[2 * blockIdx.x] = a;
    partial[2 * blockIdx.x + 1] = b;
  }
}

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 152;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 152;
  return n;
}

}  // namespace

extern "C" {

const char *oracle_cuda_last_error() { return g_error.c_str(); }

// Inversion at selected trimmed pixels (out[i] for pixels[i] = x + y width),
// over every row.  uvw [n_rows][3] metres and vis [n_rows][n_chan] complex64
// may be host or device pointers; freq, pixels and out are host memory.  No
// 1/ImageWeight, like oracle_dft_invert.  Returns 0 on success.
int oracle_cuda_dft_invert(size_t n_rows, size_t n_chan, const double *uvw, const double *freq,
                           const float *vis, size_t width, size_t height, double dl, double dm,
                           double l_shift, double m_shift, const int64_t *pixels,
                           size_t n_pixels, double *out, void *stream) {
  g_error.clear();
  cudaStream_t s = (cudaStream_t)stream;
  if (n_pixels == 0) return 0;
  if (n_rows == 0 || n_chan == 0) {
    std::memset(out, 0, sizeof(double) * n_pixels);
    return 0;
  }
  std::vector<double> lmn(3 * n_pixels);
  for (size_t i = 0; i < n_pixels; ++i)
    pixel_lmn(pixels[i], (int64_t)width, (int64_t)height, dl, dm, l_shift, m_shift, &lmn[3 * i]);
  double nu0, dnu;
  const bool lin = linear_channels(freq, n_chan, &nu0, &dnu);
  DevView d_uvw, d_vis;
  if (d_uvw.bind(uvw, sizeof(double) * 3 * n_rows, s)) return 1;
  if (d_vis.bind(vis, sizeof(float) * 2 * n_rows * n_chan, s)) return 1;
  DevArray<double> d_lmn, d_freq, d_part;
  DevArray<int> d_nc;
  if (d_lmn.alloc(3 * n_pixels) || d_freq.alloc(n_chan) || d_nc.alloc(n_rows)) return 1;
  OC_CHECK(cudaMemcpyAsync(d_lmn.ptr, lmn.data(), sizeof(double) * lmn.size(),
                           cudaMemcpyHostToDevice, s));
  OC_CHECK(cudaMemcpyAsync(d_freq.ptr, freq, sizeof(double) * n_chan, cudaMemcpyHostToDevice, s));
  row_extent_kernel<<<(unsigned)((n_rows + 255) / 256), 256, 0, s>>>(
      (const float2 *)d_vis.ptr, (int64_t)n_rows, (int)n_chan, d_nc.ptr);
  OC_CHECK(cudaGetLastError());
  const int gx = (int)((n_pixels + kThreads - 1) / kThreads);
  const int64_t want = (int64_t)sm_count() * 16;
  int64_t gy = want / gx;
  if (gy < 1) gy = 1;
  const int64_t max_gy = (int64_t)((n_rows + kRowTile - 1) / kRowTile);
  if (gy > max_gy) gy = max_gy;
  if (gy > 65535) gy = 65535;
  int64_t rpb = ((int64_t)n_rows + gy - 1) / gy;
  rpb = (rpb + kRowTile - 1) / kRowTile * kRowTile;
  gy = ((int64_t)n_rows + rpb - 1) / rpb;
  if (d_part.alloc((size_t)gy * n_pixels)) return 1;
  const size_t smem = sizeof(double2) * kRowTile * n_chan;
  if (smem > 48 * 1024)
    OC_CHECK(cudaFuncSetAttribute(dft_invert_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  dft_invert_kernel<<<dim3(gx, (unsigned)gy), kThreads, smem, s>>>(
      (const double *)d_uvw.ptr, (const float2 *)d_vis.ptr, d_nc.ptr, (int64_t)n_rows,
      (int)n_chan, rpb, d_freq.ptr, nu0 / kC, dnu / kC, lin ? 1 : 0, d_lmn.ptr, (int)n_pixels,
      d_part.ptr);
  OC_CHECK(cudaGetLastError());
  std::vector<double> part((size_t)gy * n_pixels);
  OC_CHECK(cudaMemcpyAsync(part.data(), d_part.ptr, sizeof(double) * part.size(),
                           cudaMemcpyDeviceToHost, s));
  OC_CHECK(cudaStreamSynchronize(s));
  for (size_t i = 0; i < n_pixels; ++i) {
    double a = 0.0;
    for (int64_t y = 0; y < gy; ++y) a += part[(size_t)y * n_pixels + i];
    out[i] = a;
  }
  return 0;
}

// Prediction of a trimmed model image (width x height doubles, host) at every
// sample: V = sum_p I_p e^{+2 pi i t}, like oracle_dft_predict.  uvw, mask
// ([n_rows][n_chan] bytes, nullable), pred ([n_rows][n_chan] complex64 values
// to compare, nullable) and ref_out ([n_rows][n_chan] complex128, nullable,
// written) may be host or device pointers (ref_out: device, or host memory that
// receives a copy).  sums (host) receives {sum |pred - ref|^2, sum |ref|^2}
// over the samples with mask != 0 (all samples without a mask).
int oracle_cuda_dft_predict(size_t n_rows, size_t n_chan, const double *uvw, const double *freq,
                            const double *image, size_t width, size_t height, double dl,
                            double dm, double l_shift, double m_shift, const uint8_t *mask,
                            const float *pred, double *ref_out, double *sums, void *stream) {
  g_error.clear();
  cudaStream_t s = (cudaStream_t)stream;
  sums[0] = sums[1] = 0.0;
  if (n_rows == 0 || n_chan == 0) return 0;
  std::vector<Source> src;
  for (size_t p = 0; p < width * height; ++p) {
    if (image[p] == 0.0) continue;
    Source q;
    double lmn[3];
    pixel_lmn((int64_t)p, (int64_t)width, (int64_t)height, dl, dm, l_shift, m_shift, lmn);
    q.l = lmn[0];
    q.m = lmn[1];
    q.n = lmn[2];
    q.flux = image[p];
    src.push_back(q);
  }
  double nu0, dnu;
  const bool lin = linear_channels(freq, n_chan, &nu0, &dnu);
  const size_t n = n_rows * n_chan;
  DevView d_uvw, d_mask, d_pred;
  if (d_uvw.bind(uvw, sizeof(double) * 3 * n_rows, s)) return 1;
  if (d_mask.bind(mask, n, s)) return 1;
  if (d_pred.bind(pred, sizeof(float) * 2 * n, s)) return 1;
  // ref_out: device memory is written in place, host memory through a buffer
  double2 *d_ref = nullptr;
  DevArray<double2> ref_buf;
  bool ref_host = false;
  if (ref_out) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ref_out) == cudaSuccess &&
        (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)) {
      d_ref = (double2 *)ref_out;
    } else {
      cudaGetLastError();
      if (ref_buf.alloc(n)) return 1;
      d_ref = ref_buf.ptr;
      ref_host = true;
    }
  }
  DevArray<Source> d_src;
  DevArray<double> d_freq, d_part;
  if (d_src.alloc(src.size()) || d_freq.alloc(n_chan)) return 1;
  if (!src.empty())
    OC_CHECK(cudaMemcpyAsync(d_src.ptr, src.data(), sizeof(Source) * src.size(),
                             cudaMemcpyHostToDevice, s));
  OC_CHECK(cudaMemcpyAsync(d_freq.ptr, freq, sizeof(double) * n_chan, cudaMemcpyHostToDevice, s));
  const int64_t n_cb = ((int64_t)n_chan + kChanBlock - 1) / kChanBlock;
  const int64_t n_threads = (int64_t)n_rows * n_cb;
  const int64_t blocks = (n_threads + kThreads - 1) / kThreads;
  if (d_part.alloc(2 * (size_t)blocks)) return 1;
  dft_predict_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(
      (const double *)d_uvw.ptr, (int64_t)n_rows, (int)n_chan, d_freq.ptr, dnu / kC, lin ? 1 : 0,
      d_src.ptr, (int)src.size(), (const uint8_t *)d_mask.ptr, (const float2 *)d_pred.ptr, d_ref,
      d_part.ptr);
  OC_CHECK(cudaGetLastError());
  std::vector<double> part(2 * (size_t)blocks);
  OC_CHECK(cudaMemcpyAsync(part.data(), d_part.ptr, sizeof(double) * part.size(),
                           cudaMemcpyDeviceToHost, s));
  if (ref_host)
    OC_CHECK(cudaMemcpyAsync(ref_out, d_ref, sizeof(double2) * n, cudaMemcpyDeviceToHost, s));
  OC_CHECK(cudaStreamSynchronize(s));
  for (int64_t b = 0; b < blocks; ++b) {
    sums[0] += part[2 * b];
    sums[1] += part[2 * b + 1];
  }
  return 0;
}

}  // extern "C"
