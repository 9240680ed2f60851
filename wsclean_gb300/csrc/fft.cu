// K5: shared-memory-staged 2D FFT passes, with the K4 w-screen fused into the
// column passes.
//
// A plane batch lives in HBM as [B][nv][nu] complex64.  Inversion runs
//   rows:    forward FFT of every row (length nu, one row per CTA, whole row in
//            shared memory), keeping only the `width` trimmed columns, written
//            to R = [B][nv][rstride];
//   cols A:  four-step split nv = n1 * n2: panels of 32 columns x n1 rows at
//            stride n2, forward FFT of length n1, twiddle w_nv^(r2 k1);
//   cols B:  panels of 32 columns x n2 consecutive rows, forward FFT of length
//            n2, then for every output row that maps to an image row: multiply
//            by the w-screen exp(-2 pi i w_q (n - 1 - c_n)) (FP64 argument,
//            reduced before the FP32 sincos), keep the real part, sum over the
//            planes of the batch in registers and add once into the image
//            accumulator with Kahan compensation.
// Prediction runs the adjoint passes in the opposite order (cols B', cols A',
// rows) with the opposite sign, zero padding instead of cropping.
//
// The FFT engine is a Stockham autosort with radices 2, 3, 4, 5 and 8.  Each
// stage reads every butterfly input into registers, synchronises, and writes
// the outputs in place.  Twiddles come from tables computed in FP64 on the
// host and rounded to FP32 once.
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "wgpu_internal.h"

namespace wgpu {

constexpr int kFftMaxRow = 12288;  // two row buffers fit in 227 KB of shared memory
constexpr int kMaxElemsPerThread = 16;  // complex values a thread holds per stage
constexpr int kMaxStages = 20;

int fft_row_max_length() { return kFftMaxRow; }

struct FftDesc {
  int L;
  int n_stages;
  int radix[kMaxStages];
  unsigned magic[kMaxStages];  // ceil(2^32 / p) for the stage's p
};

struct FftTables {
  std::mutex mu;
  std::map<int, float2 *> tables;
  ~FftTables() {
    for (auto &kv : tables) cudaFree(kv.second);
  }
};

FftTables *fft_tables_create() { return new FftTables(); }
void fft_tables_destroy(FftTables *t) { delete t; }

const float2 *fft_twiddles(FftTables &t, int n) {
  std::lock_guard<std::mutex> lock(t.mu);
  auto it = t.tables.find(n);
  if (it != t.tables.end()) return it->second;
  std::vector<float2> h(n);
  for (int j = 0; j < n; ++j) {
    // exp(-2 pi i j / n), argument reduced exactly in FP64
    const double a = -2.0 * M_PI * (double)j / (double)n;
    h[j] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  float2 *d = nullptr;
  WGPU_CUDA(cudaMalloc(&d, sizeof(float2) * n));
  WGPU_CUDA(cudaMemcpy(d, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
  t.tables[n] = d;
  return d;
}

static FftDesc make_desc(int L) {
  FftDesc d;
  d.L = L;
  d.n_stages = 0;
  int m = L;
  while (m % 8 == 0) { d.radix[d.n_stages++] = 8; m /= 8; }
  while (m % 4 == 0) { d.radix[d.n_stages++] = 4; m /= 4; }
  while (m % 2 == 0) { d.radix[d.n_stages++] = 2; m /= 2; }
  while (m % 3 == 0) { d.radix[d.n_stages++] = 3; m /= 3; }
  while (m % 5 == 0) { d.radix[d.n_stages++] = 5; m /= 5; }
  if (m != 1 || d.n_stages > kMaxStages)
    throw Error(WGPU_ERR_INVALID, "FFT length " + std::to_string(L) + " is not 2^a 3^b 5^c");
  unsigned long long p = 1;
  for (int st = 0; st < d.n_stages; ++st) {
    d.magic[st] = (unsigned)(((1ull << 32) + p - 1) / p);
    p *= (unsigned long long)d.radix[st];
  }
  return d;
}

namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// multiply by sign * i
__device__ __forceinline__ float2 mul_si(float2 a, float s) { return make_float2(-s * a.y, s * a.x); }

template <int R>
__device__ __forceinline__ void dft(float2 *x, float s);

template <>
__device__ __forceinline__ void dft<2>(float2 *x, float) {
  const float2 a = x[0], b = x[1];
  x[0] = cadd(a, b);
  x[1] = csub(a, b);
}

template <>
__device__ __forceinline__ void dft<4>(float2 *x, float s) {
  const float2 a = cadd(x[0], x[2]), b = csub(x[0], x[2]);
  const float2 c = cadd(x[1], x[3]), d = mul_si(csub(x[1], x[3]), s);
  x[0] = cadd(a, c);
  x[2] = csub(a, c);
  x[1] = cadd(b, d);
  x[3] = csub(b, d);
}

template <>
__device__ __forceinline__ void dft<8>(float2 *x, float s) {
  constexpr float r = 0.70710678118654752440f;
  float2 a[4], b[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    a[t] = cadd(x[t], x[t + 4]);
    b[t] = csub(x[t], x[t + 4]);
  }
  // b[t] *= exp(s 2 pi i t / 8)
  b[1] = make_float2(r * (b[1].x - s * b[1].y), r * (b[1].y + s * b[1].x));
  b[2] = mul_si(b[2], s);
  b[3] = make_float2(r * (-b[3].x - s * b[3].y), r * (-b[3].y + s * b[3].x));
  dft<4>(a, s);
  dft<4>(b, s);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    x[2 * q] = a[q];
    x[2 * q + 1] = b[q];
  }
}

template <>
__device__ __forceinline__ void dft<3>(float2 *x, float s) {
  constexpr float h = 0.86602540378443864676f;
  const float2 t1 = cadd(x[1], x[2]), t2 = csub(x[1], x[2]);
  const float2 m = make_float2(x[0].x - 0.5f * t1.x, x[0].y - 0.5f * t1.y);
  const float2 j = mul_si(make_float2(h * t2.x, h * t2.y), s);
  x[0] = cadd(x[0], t1);
  x[1] = cadd(m, j);
  x[2] = csub(m, j);
}

template <>
__device__ __forceinline__ void dft<5>(float2 *x, float s) {
  constexpr float c1 = 0.30901699437494742410f;   // cos(2 pi / 5)
  constexpr float c2 = -0.80901699437494742410f;  // cos(4 pi / 5)
  constexpr float s1 = 0.95105651629515357212f;   // sin(2 pi / 5)
  constexpr float s2 = 0.58778525229247312917f;   // sin(4 pi / 5)
  const float2 a1 = cadd(x[1], x[4]), b1 = csub(x[1], x[4]);
  const float2 a2 = cadd(x[2], x[3]), b2 = csub(x[2], x[3]);
  const float2 r1 = make_float2(x[0].x + c1 * a1.x + c2 * a2.x, x[0].y + c1 * a1.y + c2 * a2.y);
  const float2 r2 = make_float2(x[0].x + c2 * a1.x + c1 * a2.x, x[0].y + c2 * a1.y + c1 * a2.y);
  const float2 i1 = mul_si(make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y), s);
  const float2 i2 = mul_si(make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y), s);
  x[0] = cadd(x[0], cadd(a1, a2));
  x[1] = cadd(r1, i1);
  x[4] = csub(r1, i1);
  x[2] = cadd(r2, i2);
  x[3] = csub(r2, i2);
}

// Layout of the transforms a CTA holds in shared memory.
//   kRow:   one transform, element k at s[k].
//   kPanel: 32 interleaved transforms (one per column of a panel), element k
//           of transform b at s[k * 32 + b].
enum Layout { kRow = 0, kPanelLayout = 1 };

// One Stockham radix-R stage, out of place (src -> dst).  p = product of the
// radices of the earlier stages; p_magic = ceil(2^32 / p) gives i / p exactly
// for i < 2^14 (transform lengths here are at most 12288).
template <int R, Layout LAY>
__device__ __forceinline__ void stage(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                      int L, int p, unsigned p_magic, float sign,
                                      const float2 *__restrict__ tw) {
  constexpr int NB = LAY == kPanelLayout ? 32 : 1;
  const int LR = L / R;
  const int nbut = LR * NB;
  const int tw_step = L / (p * R);
  for (int u = threadIdx.x; u < nbut; u += blockDim.x) {
    const int b = LAY == kPanelLayout ? (u & 31) : 0;
    const int i = LAY == kPanelLayout ? (u >> 5) : u;
    const int k = p == 1 ? 0 : i - p * (int)__umulhi((unsigned)i, p_magic);
    float2 v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = src[(i + t * LR) * NB + b];
    if (k > 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) {
        float2 w = __ldg(tw + t * k * tw_step);
        w.y *= -sign;  // table holds exp(-2 pi i j / L); sign +1 conjugates
        v[t] = cmul(v[t], w);
      }
    }
    dft<R>(v, sign);
    const int j = (i - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) dst[(j + q * p) * NB + b] = v[q];
  }
  __syncthreads();
}

// Full transform of the data in buf[0]; buf[1] is scratch of the same size.
// sign -1 forward, +1 backward (unnormalised).  Returns the buffer holding the
// result.  The caller has synchronised after filling buf[0].
template <Layout LAY>
__device__ __forceinline__ float2 *fft_smem(float2 *buf0, float2 *buf1, const FftDesc &d,
                                            float sign, const float2 *__restrict__ tw) {
  float2 *src = buf0, *dst = buf1;
  int p = 1;
  for (int st = 0; st < d.n_stages; ++st) {
    const int R = d.radix[st];
    const unsigned m = d.magic[st];
    switch (R) {
      case 8: stage<8, LAY>(src, dst, d.L, p, m, sign, tw); break;
      case 4: stage<4, LAY>(src, dst, d.L, p, m, sign, tw); break;
      case 2: stage<2, LAY>(src, dst, d.L, p, m, sign, tw); break;
      case 3: stage<3, LAY>(src, dst, d.L, p, m, sign, tw); break;
      default: stage<5, LAY>(src, dst, d.L, p, m, sign, tw); break;
    }
    p *= R;
    float2 *t = src;
    src = dst;
    dst = t;
  }
  return src;
}

__device__ __forceinline__ int wrap(int a, int n) {
  a %= n;
  return a < 0 ? a + n : a;
}

// ---------------------------------------------------------------- rows ----
__global__ void __launch_bounds__(1024) fft_rows_forward_crop_kernel(FftDesc d, const float2 *__restrict__ planes,
                                             float2 *__restrict__ R, int rstride,
                                             int nv, int width,
                                             const float2 *__restrict__ tw) {
  extern __shared__ float2 s[];
  const int L = d.L;
  const size_t row = blockIdx.x;  // plane * nv + b
  const float2 *src = planes + row * (size_t)L;
  for (int k = threadIdx.x; k < L / 2; k += blockDim.x)
    reinterpret_cast<float4 *>(s)[k] = __ldg(reinterpret_cast<const float4 *>(src) + k);
  __syncthreads();
  const float2 *res = fft_smem<kRow>(s, s + L, d, -1.0f, tw);
  float2 *dst = R + row * (size_t)rstride;
  for (int x = threadIdx.x; x < rstride; x += blockDim.x) {
    float2 v = make_float2(0.f, 0.f);
    if (x < width) v = res[wrap(width / 2 - x, L)];
    dst[x] = v;
  }
}

__global__ void __launch_bounds__(1024) fft_rows_backward_pad_kernel(FftDesc d, const float2 *__restrict__ R,
                                             int rstride, float2 *__restrict__ planes,
                                             int nv, int width,
                                             const float2 *__restrict__ tw) {
  extern __shared__ float2 s[];
  const int L = d.L;
  const size_t row = blockIdx.x;
  for (int k = threadIdx.x; k < L; k += blockDim.x) s[k] = make_float2(0.f, 0.f);
  __syncthreads();
  const float2 *src = R + row * (size_t)rstride;
  for (int x = threadIdx.x; x < width; x += blockDim.x) s[wrap(width / 2 - x, L)] = src[x];
  __syncthreads();
  const float2 *res = fft_smem<kRow>(s, s + L, d, +1.0f, tw);
  float2 *dst = planes + row * (size_t)L;
  for (int k = threadIdx.x; k < L / 2; k += blockDim.x)
    reinterpret_cast<float4 *>(dst)[k] = reinterpret_cast<const float4 *>(res)[k];
}

// ------------------------------------------------------------- columns ----
constexpr int kColThreads = 512;
constexpr int kPanel = 32;  // columns per panel

// Pass A (forward) / A' (backward): strided length-n1 transforms.
__global__ void __launch_bounds__(kColThreads)
    fft_cols_pass_a_kernel(FftDesc d1, float2 *__restrict__ R, int rstride, int nv,
                           int n2, float sign, const float2 *__restrict__ tw1,
                           const float2 *__restrict__ twN) {
  extern __shared__ float2 s[];
  const int n1 = d1.L;
  const int cg = blockIdx.x, r2 = blockIdx.y;
  float2 *base = R + (size_t)blockIdx.z * nv * rstride + cg * kPanel;
  for (int e = threadIdx.x; e < n1 * kPanel; e += blockDim.x) {
    const int r1 = e / kPanel, c = e % kPanel;
    s[e] = base[(size_t)(r2 + n2 * r1) * rstride + c];
  }
  __syncthreads();
  // backward: this pass runs last and the twiddle was applied in pass B'
  const float2 *res = fft_smem<kPanelLayout>(s, s + n1 * kPanel, d1, sign, tw1);
  for (int e = threadIdx.x; e < n1 * kPanel; e += blockDim.x) {
    const int k1 = e / kPanel, c = e % kPanel;
    float2 v = res[e];
    if (sign < 0) v = cmul(v, __ldg(twN + (int)(((long long)r2 * k1) % nv)));
    base[(size_t)(r2 + n2 * k1) * rstride + c] = v;
  }
}

__device__ __forceinline__ int image_row_of(int k, int nv, int height) {
  // FFT output index k holds Y = k (k < height/2) or Y = k - nv
  // (k >= nv - height/2); image row y = Y + height/2.
  const int hh = height / 2;
  if (k < hh) return k + hh;
  if (k >= nv - hh) return k - nv + hh;
  return -1;
}

__device__ __forceinline__ void screen(double wq, double nu, float *s, float *c) {
  double t = wq * nu;
  t -= rint(t);
  sincospif(2.0f * (float)t, s, c);
}

// Pass B (forward) with the fused w-screen and accumulation over the batch.
__global__ void __launch_bounds__(kColThreads)
    fft_cols_forward_accumulate_kernel(FftDesc d2, DevPlan p, int n1,
                                       float2 *__restrict__ R, int rstride,
                                       int n_batch, int p_begin,
                                       const double *__restrict__ nu_w,
                                       float2 *__restrict__ acc,
                                       const float2 *__restrict__ tw2) {
  extern __shared__ float2 s[];
  const int n2 = d2.L;
  const int nv = p.nv;
  const int cg = blockIdx.x, k1 = blockIdx.y;
  constexpr int NE = kMaxElemsPerThread;
  float part[NE];
#pragma unroll
  for (int c = 0; c < NE; ++c) part[c] = 0.f;
  for (int b = 0; b < n_batch; ++b) {
    const float2 *base = R + (size_t)b * nv * rstride + (size_t)n2 * k1 * rstride + cg * kPanel;
    for (int e = threadIdx.x; e < n2 * kPanel; e += blockDim.x) {
      const int r2 = e / kPanel, c = e % kPanel;
      s[e] = base[(size_t)r2 * rstride + c];
    }
    __syncthreads();
    const float2 *res = fft_smem<kPanelLayout>(s, s + n2 * kPanel, d2, -1.0f, tw2);
    const double wq = p.w0 + (double)(p_begin + b) * p.dw;
#pragma unroll
    for (int c = 0; c < NE; ++c) {
      const int e = threadIdx.x + c * blockDim.x;
      if (e < n2 * kPanel) {
        const int k2 = e / kPanel, col = e % kPanel;
        const int x = cg * kPanel + col;
        const int y = image_row_of(k1 + n1 * k2, nv, p.height);
        if (x < p.width && y >= 0) {
          const float2 v = res[e];
          float sn, cs;
          screen(wq, __ldg(nu_w + (size_t)y * p.width + x), &sn, &cs);
          // Re(v exp(-2 pi i t)) = v.re cos + v.im sin
          part[c] += v.x * cs + v.y * sn;
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int c = 0; c < NE; ++c) {
    const int e = threadIdx.x + c * blockDim.x;
    if (e < n2 * kPanel) {
      const int k2 = e / kPanel, col = e % kPanel;
      const int x = cg * kPanel + col;
      const int y = image_row_of(k1 + n1 * k2, nv, p.height);
      if (x < p.width && y >= 0) {
        float2 *a = acc + (size_t)y * p.width + x;
        float2 sc = *a;  // (sum, compensation)
        const float yv = part[c] - sc.y;
        const float t = sc.x + yv;
        sc.y = (t - sc.x) - yv;
        sc.x = t;
        *a = sc;
      }
    }
  }
}

// Pass B' (backward): screened, pre-corrected image rows -> length-n2
// backward transforms -> twiddle -> R rows n2*k1 + r2.
__global__ void __launch_bounds__(kColThreads)
    fft_cols_backward_screen_kernel(FftDesc d2, DevPlan p, int n1,
                                    const float *__restrict__ img_corr,
                                    const double *__restrict__ nu_w,
                                    float2 *__restrict__ R, int rstride,
                                    int n_batch, int p_begin,
                                    const float2 *__restrict__ tw2,
                                    const float2 *__restrict__ twN) {
  extern __shared__ float2 s[];
  const int n2 = d2.L;
  const int nv = p.nv;
  const int cg = blockIdx.x, k1 = blockIdx.y;
  for (int b = 0; b < n_batch; ++b) {
    const double wq = p.w0 + (double)(p_begin + b) * p.dw;
    for (int e = threadIdx.x; e < n2 * kPanel; e += blockDim.x) {
      const int k2 = e / kPanel, col = e % kPanel;
      const int x = cg * kPanel + col;
      const int y = image_row_of(k1 + n1 * k2, nv, p.height);
      float2 v = make_float2(0.f, 0.f);
      if (x < p.width && y >= 0) {
        const size_t i = (size_t)y * p.width + x;
        const float a = __ldg(img_corr + i);
        if (a != 0.0f) {
          float sn, cs;
          screen(wq, __ldg(nu_w + i), &sn, &cs);
          // a exp(+2 pi i t)
          v = make_float2(a * cs, a * sn);
        }
      }
      s[e] = v;
    }
    __syncthreads();
    const float2 *res = fft_smem<kPanelLayout>(s, s + n2 * kPanel, d2, +1.0f, tw2);
    float2 *base = R + (size_t)b * nv * rstride + (size_t)n2 * k1 * rstride + cg * kPanel;
    for (int e = threadIdx.x; e < n2 * kPanel; e += blockDim.x) {
      const int r2 = e / kPanel, c = e % kPanel;
      float2 v = res[e];
      if (n1 > 1) {
        float2 w = __ldg(twN + (int)(((long long)r2 * k1) % nv));
        w.y = -w.y;  // exp(+2 pi i r2 k1 / nv)
        v = cmul(v, w);
      }
      base[(size_t)r2 * rstride + c] = v;
    }
    __syncthreads();
  }
}

// Threads for a row transform of length L (about L/8 butterflies per stage).
int row_threads(int L) {
  int t = (L / 8 + 31) / 32 * 32;
  return t < 64 ? 64 : (t > 1024 ? 1024 : t);
}

void set_smem(const void *fn, size_t bytes) { ensure_dynamic_smem(fn, bytes); }

}  // namespace

void launch_fft_rows_forward_crop(FftTables &t, const DevPlan &p,
                                  const float2 *planes, float2 *R, int rstride,
                                  int n_batch, cudaStream_t s) {
  const FftDesc d = make_desc(p.nu);
  const float2 *tw = fft_twiddles(t, p.nu);
  const size_t smem = 2 * sizeof(float2) * p.nu;
  set_smem((const void *)fft_rows_forward_crop_kernel, smem);
  fft_rows_forward_crop_kernel<<<(unsigned)((size_t)n_batch * p.nv), row_threads(p.nu), smem, s>>>(
      d, planes, R, rstride, p.nv, p.width, tw);
  check_launch("fft_rows_forward_crop_kernel");
}

void launch_fft_rows_backward_pad(FftTables &t, const DevPlan &p,
                                  const float2 *R, int rstride, float2 *planes,
                                  int n_batch, cudaStream_t s) {
  const FftDesc d = make_desc(p.nu);
  const float2 *tw = fft_twiddles(t, p.nu);
  const size_t smem = 2 * sizeof(float2) * p.nu;
  set_smem((const void *)fft_rows_backward_pad_kernel, smem);
  fft_rows_backward_pad_kernel<<<(unsigned)((size_t)n_batch * p.nv), row_threads(p.nu), smem, s>>>(
      d, R, rstride, planes, p.nv, p.width, tw);
  check_launch("fft_rows_backward_pad_kernel");
}

void launch_fft_cols_a(FftTables &t, const DevPlan &p, int n1, int n2, float2 *R,
                       int rstride, int n_batch, float sign, cudaStream_t s) {
  if (n1 <= 1) return;
  const int ncg = rstride / kPanel;
  const FftDesc d1 = make_desc(n1);
  const size_t smem = 2 * sizeof(float2) * n1 * kPanel;
  set_smem((const void *)fft_cols_pass_a_kernel, smem);
  dim3 grid(ncg, n2, n_batch);
  fft_cols_pass_a_kernel<<<grid, kColThreads, smem, s>>>(
      d1, R, rstride, p.nv, n2, sign, fft_twiddles(t, n1), fft_twiddles(t, p.nv));
  check_launch("fft_cols_pass_a_kernel");
}

void launch_fft_cols_b_forward_accumulate(FftTables &t, const DevPlan &p, int n1,
                                          int n2, float2 *R, int rstride,
                                          int n_batch, int p_begin,
                                          const double *nu_w, float2 *acc,
                                          cudaStream_t s) {
  const int ncg = rstride / kPanel;
  const FftDesc d2 = make_desc(n2);
  const size_t smem = 2 * sizeof(float2) * n2 * kPanel;
  set_smem((const void *)fft_cols_forward_accumulate_kernel, smem);
  dim3 grid(ncg, n1);
  fft_cols_forward_accumulate_kernel<<<grid, kColThreads, smem, s>>>(
      d2, p, n1, R, rstride, n_batch, p_begin, nu_w, acc, fft_twiddles(t, n2));
  check_launch("fft_cols_forward_accumulate_kernel");
}

void launch_fft_cols_b_backward_screen(FftTables &t, const DevPlan &p, int n1,
                                       int n2, const float *img_corr,
                                       const double *nu_w, float2 *R,
                                       int rstride, int n_batch, int p_begin,
                                       cudaStream_t s) {
  const int ncg = rstride / kPanel;
  const FftDesc d2 = make_desc(n2);
  const size_t smem = 2 * sizeof(float2) * n2 * kPanel;
  set_smem((const void *)fft_cols_backward_screen_kernel, smem);
  dim3 grid(ncg, n1);
  fft_cols_backward_screen_kernel<<<grid, kColThreads, smem, s>>>(
      d2, p, n1, img_corr, nu_w, R, rstride, n_batch, p_begin,
      fft_twiddles(t, n2), fft_twiddles(t, p.nv));
  check_launch("fft_cols_backward_screen_kernel");
}

}  // namespace wgpu
