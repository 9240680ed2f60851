// K5: shared-memory-staged 2D FFT passes, with the K4 w-screen fused into the
// column passes.
//
// A plane batch lives in HBM as [B][nv][nu] complex64.  Inversion runs
//   rows:    forward FFT of every row that some footprint touches (the row
//            list of the bucketing pass; length nu, whole row in shared
//            memory), keeping only the `width` trimmed columns, written to
//            R = [B][nv][rstride];
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
// The FFT engine is a Stockham autosort with radices 2, 3, 4, 5, 6, 8 and 16.
// Row stages read every butterfly input into registers, synchronise, and write
// the outputs in place.  Column transforms of length 16 R2 (R2 in 2, 3, 4, 5,
// 6, 8) take two stages with one shared-memory round trip (panel_fft); other
// lengths use the generic stage loop.  Twiddles come from tables computed in
// FP64 on the host and rounded to FP32 once.
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "screen.cuh"
#include "tma.cuh"
#include "wgpu_internal.h"

namespace wgpu {

constexpr int kFftMaxRow = 12288;  // two row buffers fit in 227 KB of shared memory
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
  std::map<int, float2 *> tables;      // exp(-2 pi i j / n), j < n
  std::map<int, float2 *> row_tables;  // per-stage tables of row schedules
  ~FftTables() {
    for (auto &kv : tables) cudaFree(kv.second);
    for (auto &kv : row_tables) cudaFree(kv.second);
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

// Radix schedule for length L: radix 16 first where allowed (row transforms;
// the later strides are then multiples of 16, which with the row swizzle
// keeps every stage free of bank conflicts), then 8, 4, 2, 3, 5.
static FftDesc make_desc(int L, bool radix16 = false) {
  FftDesc d;
  d.L = L;
  d.n_stages = 0;
  int m = L;
  if (radix16)
    while (m % 16 == 0) { d.radix[d.n_stages++] = 16; m /= 16; }
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

// 16 = 4 x 4: DFT4 over n1 of x[4 n1 + n2], twiddle w16^(n2 k1), DFT4 over
// n2; output k1 + 4 k2.
template <>
__device__ __forceinline__ void dft<16>(float2 *x, float s) {
  constexpr float c8 = 0.92387953251128675613f;  // cos(pi / 8)
  constexpr float s8 = 0.38268343236508977173f;  // sin(pi / 8)
  constexpr float r = 0.70710678118654752440f;
  float2 y[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) y[n2][n1] = x[4 * n1 + n2];
    dft<4>(y[n2], s);
  }
  // w16^e = exp(s 2 pi i e / 16) for e = n2 k1
  const float2 w1 = make_float2(c8, s * s8), w2 = make_float2(r, s * r),
               w3 = make_float2(s8, s * c8), w6 = make_float2(-r, s * r),
               w9 = make_float2(-c8, -s * s8);
  y[1][1] = cmul(y[1][1], w1);
  y[1][2] = cmul(y[1][2], w2);
  y[1][3] = cmul(y[1][3], w3);
  y[2][1] = cmul(y[2][1], w2);
  y[2][2] = mul_si(y[2][2], s);
  y[2][3] = cmul(y[2][3], w6);
  y[3][1] = cmul(y[3][1], w3);
  y[3][2] = cmul(y[3][2], w6);
  y[3][3] = cmul(y[3][3], w9);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 z[4];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) z[n2] = y[n2][k1];
    dft<4>(z, s);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) x[k1 + 4 * k2] = z[k2];
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

// 6 = 2 x 3: E = DFT3 of the even inputs, O of the odd ones; X[k] = E[k] +
// w6^k O[k], X[k + 3] = E[k] - w6^k O[k] (k < 3), w6 = exp(s 2 pi i / 6).
template <>
__device__ __forceinline__ void dft<6>(float2 *x, float s) {
  constexpr float h = 0.86602540378443864676f;  // sin(pi / 3)
  float2 e[3] = {x[0], x[2], x[4]}, o[3] = {x[1], x[3], x[5]};
  dft<3>(e, s);
  dft<3>(o, s);
  const float2 o1 = make_float2(0.5f * o[1].x - s * h * o[1].y, 0.5f * o[1].y + s * h * o[1].x);
  const float2 o2 = make_float2(-0.5f * o[2].x - s * h * o[2].y, -0.5f * o[2].y + s * h * o[2].x);
  x[0] = cadd(e[0], o[0]);
  x[3] = csub(e[0], o[0]);
  x[1] = cadd(e[1], o1);
  x[4] = csub(e[1], o1);
  x[2] = cadd(e[2], o2);
  x[5] = csub(e[2], o2);
}

// Layout of the transforms a CTA holds in shared memory.
//   kRow:   one transform, element k at s[row_slot(k)]: the low four bits of
//           k are XORed with bits 4-7, which puts the strided accesses of
//           every stage (and the natural-order fill and read-out) on distinct
//           banks.  Buffers are rounded up to a multiple of 16 elements.
//   kPanel: 32 interleaved transforms (one per column of a panel), element k
//           of transform b at s[k * 32 + b].
enum Layout { kRow = 0, kPanelLayout = 1 };

__device__ __forceinline__ int row_slot(int k) { return k ^ ((k >> 4) & 15); }
__host__ __device__ constexpr int row_buffer(int L) { return (L + 15) & ~15; }

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
    for (int t = 0; t < R; ++t)
      v[t] = LAY == kRow ? src[row_slot(i + t * LR)] : src[(i + t * LR) * NB + b];
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
    for (int q = 0; q < R; ++q) {
      if (LAY == kRow)
        dst[row_slot(j + q * p)] = v[q];
      else
        dst[(j + q * p) * NB + b] = v[q];
    }
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
      case 16:
        if constexpr (LAY == kRow) stage<16, LAY>(src, dst, d.L, p, m, sign, tw);
        break;
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
// Row transforms (length L = nu, a multiple of 16) use radix 16 first and the
// swizzled row layout; twiddles come from per-stage tables laid out
// [t - 1][k] (exp(-2 pi i t k / (p R))), so the lanes of a warp (consecutive
// k) read consecutive entries.  Two kernels:
//  * rows longer than kRowPingPongMax (8192, 10240, 12288): a persistent
//    kernel, one CTA per SM looping over rows; the transform runs in place in
//    one buffer (each thread holds the inputs of its butterflies in registers
//    across a barrier) while a TMA bulk copy (cp.async.bulk, completion on an
//    mbarrier) brings the next row into the other buffer.
//  * shorter rows: one CTA per row, Stockham stages ping-ponging between two
//    buffers, L / 16 threads, several CTAs per SM.

constexpr int kRowPingPongMax = 6912;
constexpr int kRowIn = 0;      // stage input: natural order as copied
constexpr int kRowInPad = 1;   // natural order of the zero-padded, re-centred row
constexpr int kRowInSlot = 2;  // swizzled layout written by an earlier stage

struct RowStages {
  int tw_off[kMaxStages];  // offset of each stage's table in the row table
};

// Self-test of the bounded wait: waits on an mbarrier that nothing arrives
// at, so the wait must expire; records the expiry and returns.
__global__ void bounded_wait_selftest_kernel(long long cycles, unsigned *err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar);
  __syncthreads();
  const bool ok = mbar_wait_bounded(&bar, 0, cycles);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicAdd(err, 1u);
}

// Loads element a of the stage input.
template <int IN>
__device__ __forceinline__ float2 row_in(const float2 *buf, int a, int L, int width) {
  if (IN == kRowIn) return buf[a];
  if (IN == kRowInPad) {
    const int x = wrap(width / 2 - a, L);
    return x < width ? buf[x] : make_float2(0.f, 0.f);
  }
  return buf[row_slot(a)];
}

// Stockham butterfly i of a radix-R stage: twiddle, DFT, outputs in v.
template <int R>
__device__ __forceinline__ int row_butterfly(float2 *v, int i, int p, unsigned p_magic, float sign,
                                             const float2 *__restrict__ tws) {
  const int k = p == 1 ? 0 : i - p * (int)__umulhi((unsigned)i, p_magic);
  if (k > 0) {
#pragma unroll
    for (int t = 1; t < R; ++t) {
      float2 w = tws[(t - 1) * p + k];  // shared or read-only global table
      w.y *= -sign;  // tables hold exp(-2 pi i t k / (p R)); sign +1 conjugates
      v[t] = cmul(v[t], w);
    }
  }
  dft<R>(v, sign);
  return (i - k) * R + k;  // outputs go to j + q p
}

// One in-place Stockham stage of radix R over buf (length L).  blockDim.x >=
// L / 16, so a thread holds at most ceil(16 / R) butterflies.
template <int R, int IN>
__device__ __forceinline__ void row_stage_inplace(float2 *buf, int L, int p, unsigned p_magic,
                                                  float sign, const float2 *__restrict__ tws,
                                                  int width) {
  constexpr int KMAX = (16 + R - 1) / R;
  const int LR = L / R;
  float2 v[KMAX][R];
#pragma unroll
  for (int kk = 0; kk < KMAX; ++kk) {
    const int i = threadIdx.x + kk * blockDim.x;
    if (i < LR) {
#pragma unroll
      for (int t = 0; t < R; ++t) v[kk][t] = row_in<IN>(buf, i + t * LR, L, width);
    }
  }
  __syncthreads();
#pragma unroll
  for (int kk = 0; kk < KMAX; ++kk) {
    const int i = threadIdx.x + kk * blockDim.x;
    if (i < LR) {
      const int j = row_butterfly<R>(v[kk], i, p, p_magic, sign, tws);
#pragma unroll
      for (int q = 0; q < R; ++q) buf[row_slot(j + q * p)] = v[kk][q];
    }
  }
  __syncthreads();
}

// Last stage with its outputs written straight to the output row (no
// shared-memory write and read-out): output k goes to column
// x = (width/2 - k) mod L when x < width (FWD: the kept, re-centred columns;
// columns width .. out_stride - 1 are zero) or to position k (!FWD).
template <int R, bool FWD>
__device__ __forceinline__ void row_stage_last_out(const float2 *buf, int L, int p, float sign,
                                                   const float2 *__restrict__ tws,
                                                   float2 *__restrict__ out, int out_stride,
                                                   int width) {
  const int LR = L / R;  // == p
  for (int i = threadIdx.x; i < LR; i += blockDim.x) {
    float2 v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = buf[row_slot(i + t * LR)];
    if (i > 0) {
#pragma unroll
      for (int t = 1; t < R; ++t) {
        float2 w = __ldg(tws + (t - 1) * p + i);
        w.y *= -sign;
        v[t] = cmul(v[t], w);
      }
    }
    dft<R>(v, sign);
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int k = i + q * LR;
      if (FWD) {
        int x = width / 2 - k;
        if (x < 0) x += L;
        if (x < width) out[x] = v[q];
      } else {
        out[k] = v[q];
      }
    }
  }
  if (FWD)
    for (int x = width + threadIdx.x; x < out_stride; x += blockDim.x)
      out[x] = make_float2(0.f, 0.f);
}

// Writes the transformed row: FWD crops the `width` kept columns (re-centred)
// into out (out_stride entries), !FWD writes the L entries in natural order.
template <bool FWD>
__device__ __forceinline__ void row_out(const float2 *res, float2 *__restrict__ out,
                                        int out_stride, int L, int width) {
  float4 *dst = reinterpret_cast<float4 *>(out);
  if (FWD) {
    for (int x2 = threadIdx.x; x2 < out_stride / 2; x2 += blockDim.x) {
      const int x = 2 * x2;
      const float2 a = x < width ? res[row_slot(wrap(width / 2 - x, L))] : make_float2(0.f, 0.f);
      const float2 c =
          x + 1 < width ? res[row_slot(wrap(width / 2 - x - 1, L))] : make_float2(0.f, 0.f);
      dst[x2] = make_float4(a.x, a.y, c.x, c.y);
    }
  } else {
    for (int k2 = threadIdx.x; k2 < L / 2; k2 += blockDim.x) {
      const float2 a = res[row_slot(2 * k2)], c = res[row_slot(2 * k2 + 1)];
      dst[k2] = make_float4(a.x, a.y, c.x, c.y);
    }
  }
}

constexpr int kRowThreadsMax = kFftMaxRow / 16;  // 768: one radix-16 butterfly each

// Number of rows a row launch transforms, and the batch row index of its
// item idx (see RowSel).
__device__ __forceinline__ int sel_rows(const RowSel &sel, int n_batch, int nv) {
  return sel.list ? (int)(__ldg(sel.start + n_batch) - __ldg(sel.start)) : n_batch * nv;
}
__device__ __forceinline__ int sel_row(const RowSel &sel, int idx, int nv) {
  return sel.list ? (int)(__ldg(sel.list + __ldg(sel.start) + idx) - (uint32_t)sel.p_begin * nv)
                  : idx;
}

// Persistent row kernel.  Schedule: radix 16, (n_stages - 2 - MID8) radix-16
// stages, one radix-8 stage if MID8, and a last stage of radix LAST that
// writes straight to the output row.
// FWD: plane rows (length L) -> forward FFT -> cropped rows of R.
// !FWD: rows of R (width valid entries) -> zero padding, re-centring ->
//      backward FFT -> plane rows.  buf_elems >= max(L, in_stride); in_bytes
// is the size of one input row.  Only the rows `sel` names are transformed.
template <bool FWD, int LAST, bool MID8>
__global__ void __launch_bounds__(kRowThreadsMax, 1)
    fft_rows_persistent_kernel(FftDesc d, RowStages st, const float2 *__restrict__ tws,
                               const float2 *__restrict__ in, int in_stride, uint32_t in_bytes,
                               float2 *__restrict__ out, int out_stride, int n_batch, int nv,
                               RowSel sel, int width, int buf_elems, int mid_tab,
                               unsigned *__restrict__ err) {
  extern __shared__ __align__(128) unsigned char row_smem[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(row_smem);  // two mbarriers
  float2 *bufs = reinterpret_cast<float2 *>(row_smem + 128);
  // twiddles of the middle stages (mid_tab entries from stage 1 on), copied
  // once per CTA when they fit; otherwise read from global memory
  float2 *tab = bufs + 2 * (size_t)buf_elems;
  const int L = d.L;
  const float sign = FWD ? -1.0f : 1.0f;
  const int G = gridDim.x;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0]);
    mbar_init(&bar[1]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_proxy_async();
  }
  for (int i = threadIdx.x; i < mid_tab; i += blockDim.x) tab[i] = __ldg(tws + st.tw_off[1] + i);
  __syncthreads();
  const int n_items = sel_rows(sel, n_batch, nv);
  int item = blockIdx.x;
  if (threadIdx.x == 0 && item < n_items) {
    mbar_expect_tx(&bar[0], in_bytes);
    bulk_copy_g2s(bufs, in + (size_t)sel_row(sel, item, nv) * in_stride, in_bytes, &bar[0]);
  }
  uint32_t phase0 = 0, phase1 = 0;
  for (int it = 0; item < n_items; ++it, item += G) {
    const int b = it & 1;
    float2 *buf = bufs + (size_t)b * buf_elems;
    const int row = sel_row(sel, item, nv);
    const int next = item + G;
    if (next < n_items && threadIdx.x == 0) {
      mbar_expect_tx(&bar[b ^ 1], in_bytes);
      bulk_copy_g2s(bufs + (size_t)(b ^ 1) * buf_elems,
                    in + (size_t)sel_row(sel, next, nv) * in_stride, in_bytes, &bar[b ^ 1]);
    }
    const bool ok = mbar_wait_bounded(&bar[b], b == 0 ? phase0 : phase1);
    if (__syncthreads_or(!ok)) {
      // a copy did not complete in time: record it, wait once more (bounded)
      // for the copies still in flight, and leave
      if (threadIdx.x == 0) atomicAdd(err, 1u);
      mbar_wait_bounded(&bar[b], b == 0 ? phase0 : phase1);
      if (next < n_items) mbar_wait_bounded(&bar[b ^ 1], b == 0 ? phase1 : phase0);
      return;
    }
    if (b == 0) phase0 ^= 1; else phase1 ^= 1;
    row_stage_inplace<16, FWD ? kRowIn : kRowInPad>(buf, L, 1, d.magic[0], sign,
                                                     tws + st.tw_off[0], width);
    int p = 16, s = 1;
    const int n_mid16 = d.n_stages - 2 - (MID8 ? 1 : 0);
    for (int m = 0; m < n_mid16; ++m, ++s) {
      const float2 *tw = mid_tab ? tab + (st.tw_off[s] - st.tw_off[1]) : tws + st.tw_off[s];
      row_stage_inplace<16, kRowInSlot>(buf, L, p, d.magic[s], sign, tw, width);
      p *= 16;
    }
    if (MID8) {
      const float2 *tw = mid_tab ? tab + (st.tw_off[s] - st.tw_off[1]) : tws + st.tw_off[s];
      row_stage_inplace<8, kRowInSlot>(buf, L, p, d.magic[s], sign, tw, width);
      p *= 8;
      ++s;
    }
    row_stage_last_out<LAST, FWD>(buf, L, p, sign, tws + st.tw_off[s],
                                  out + (size_t)row * out_stride, out_stride, width);
    // generic accesses to this buffer end here; the bulk copy issued into it
    // at the next iteration is ordered after them
    fence_proxy_async();
    __syncthreads();
  }
}

// Out-of-place Stockham stage over the swizzled row layout.
template <int R>
__device__ __forceinline__ void row_stage_pp(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                             int L, int p, unsigned p_magic, float sign,
                                             const float2 *__restrict__ tws) {
  const int LR = L / R;
  for (int i = threadIdx.x; i < LR; i += blockDim.x) {
    float2 v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = src[row_slot(i + t * LR)];
    const int j = row_butterfly<R>(v, i, p, p_magic, sign, tws);
#pragma unroll
    for (int q = 0; q < R; ++q) dst[row_slot(j + q * p)] = v[q];
  }
  __syncthreads();
}

// Ping-pong row kernel, one CTA per row (rows up to kRowPingPongMax), launched
// with L / 16 threads rounded up to whole warps, at most kRowPingPongThreads
// (every loop of the kernel strides by blockDim.x, and no warp-wide
// intrinsic is used, so the last warp may be partial).
constexpr int kRowPingPongThreads = kRowPingPongMax / 16;
template <bool FWD>
__global__ void __launch_bounds__(kRowPingPongThreads, 2)
    fft_rows_pingpong_kernel(FftDesc d, RowStages st, const float2 *__restrict__ tws,
                             const float2 *__restrict__ in, int in_stride,
                             float2 *__restrict__ out, int out_stride, int n_batch, int nv,
                             RowSel sel, int width) {
  extern __shared__ float2 s[];
  const int L = d.L;
  const float sign = FWD ? -1.0f : 1.0f;
  if ((int)blockIdx.x >= sel_rows(sel, n_batch, nv)) return;  // whole block
  const size_t row = (size_t)sel_row(sel, blockIdx.x, nv);
  float2 *buf0 = s, *buf1 = s + row_buffer(L);
  if (FWD) {
    const float4 *src = reinterpret_cast<const float4 *>(in + row * in_stride);
    for (int k = threadIdx.x; k < L / 2; k += blockDim.x) {
      const float4 v = __ldg(src + k);
      buf0[row_slot(2 * k)] = make_float2(v.x, v.y);
      buf0[row_slot(2 * k + 1)] = make_float2(v.z, v.w);
    }
  } else {
    for (int k = threadIdx.x; k < L; k += blockDim.x) buf0[k] = make_float2(0.f, 0.f);
    __syncthreads();
    const float2 *src = in + row * in_stride;
    for (int x = threadIdx.x; x < width; x += blockDim.x)
      buf0[row_slot(wrap(width / 2 - x, L))] = __ldg(src + x);
  }
  __syncthreads();
  float2 *a = buf0, *b = buf1;
  int p = 1;
  for (int st_i = 0; st_i < d.n_stages; ++st_i) {
    const float2 *tw = tws + st.tw_off[st_i];
    switch (d.radix[st_i]) {
      case 16: row_stage_pp<16>(a, b, L, p, d.magic[st_i], sign, tw); break;
      case 8: row_stage_pp<8>(a, b, L, p, d.magic[st_i], sign, tw); break;
      case 4: row_stage_pp<4>(a, b, L, p, d.magic[st_i], sign, tw); break;
      case 2: row_stage_pp<2>(a, b, L, p, d.magic[st_i], sign, tw); break;
      case 3: row_stage_pp<3>(a, b, L, p, d.magic[st_i], sign, tw); break;
      default: row_stage_pp<5>(a, b, L, p, d.magic[st_i], sign, tw); break;
    }
    p *= d.radix[st_i];
    float2 *t = a;
    a = b;
    b = t;
  }
  row_out<FWD>(a, out + row * out_stride, out_stride, L, width);
}

// ------------------------------------------------------------- columns ----
constexpr int kColThreads = 512;
constexpr int kPanel = 32;  // columns per panel

// Loads a panel of n_rows x kPanel elements (row r at src + r * row_stride)
// into shared memory, issuing all of a thread's loads before the stores so
// that enough bytes are in flight to cover the HBM latency.
// With row_flags, panel row r is read only where row_flags[r * flag_stride]
// is set and is zero elsewhere.
__device__ __forceinline__ void load_panel(float2 *__restrict__ s, const float2 *__restrict__ src,
                                           size_t row_stride, int n_rows,
                                           const uint8_t *__restrict__ row_flags = nullptr,
                                           int flag_stride = 0) {
  constexpr int kBatch = 8;  // loads in flight per thread
  const int n_el = n_rows * kPanel;
  for (int e0 = threadIdx.x; e0 < n_el; e0 += kBatch * blockDim.x) {
    float2 tmp[kBatch];
#pragma unroll
    for (int k = 0; k < kBatch; ++k) {
      const int e = e0 + k * blockDim.x;
      if (e < n_el) {
        const int r = e / kPanel;
        tmp[k] = (!row_flags || __ldg(row_flags + (size_t)r * flag_stride))
                     ? __ldg(src + (size_t)r * row_stride + (e % kPanel))
                     : make_float2(0.f, 0.f);
      }
    }
#pragma unroll
    for (int k = 0; k < kBatch; ++k) {
      const int e = e0 + k * blockDim.x;
      if (e < n_el) s[e] = tmp[k];
    }
  }
}

// Pass A (forward) / A' (backward): strided length-n1 transforms.
__global__ void __launch_bounds__(kColThreads, 3)
    fft_cols_pass_a_kernel(FftDesc d1, float2 *__restrict__ R, int rstride, int nv,
                           int n2, float sign, const float2 *__restrict__ tw1,
                           const float2 *__restrict__ twN, const uint8_t *__restrict__ flags) {
  extern __shared__ float2 s[];
  const int n1 = d1.L;
  const int cg = blockIdx.x, r2 = blockIdx.y;
  float2 *base = R + (size_t)blockIdx.z * nv * rstride + cg * kPanel;
  // flags of this plane's rows (null: every row carries data)
  const uint8_t *fl = flags ? flags + (size_t)blockIdx.z * nv : nullptr;
  if (sign < 0)
    load_panel(s, base + (size_t)r2 * rstride, (size_t)n2 * rstride, n1, fl ? fl + r2 : nullptr,
               n2);
  else
    load_panel(s, base + (size_t)r2 * rstride, (size_t)n2 * rstride, n1);
  __syncthreads();
  // backward: this pass runs last and the twiddle was applied in pass B'
  const float2 *res = fft_smem<kPanelLayout>(s, s + n1 * kPanel, d1, sign, tw1);
  for (int e = threadIdx.x; e < n1 * kPanel; e += blockDim.x) {
    const int k1 = e / kPanel, c = e % kPanel;
    float2 v = res[e];
    // r2 < n2 and k1 < n1, so r2 k1 < nv indexes the table directly
    if (sign < 0) v = cmul(v, __ldg(twN + r2 * k1));
    // backward: rows no visibility reads are not written
    if (sign < 0 || !fl || __ldg(fl + r2 + n2 * k1)) base[(size_t)(r2 + n2 * k1) * rstride + c] = v;
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

// The w-screen of plane q at a pixel from its screen terms (screen.cuh).
constexpr float kNoPixel = 8.0f;  // remainder marker of panel elements outside the image
__device__ __forceinline__ void screen_b(uint32_t a, uint32_t k, float r, int q, float *sn,
                                         float *cs) {
  sincospif(screen_arg2(a, k, r, q), sn, cs);
}

// Shared layout of the column-B kernels: the two FFT buffers (n2 * kPanel
// each), then the per-element screen terms a, k, r (n2 * kPanel each).
__host__ __device__ constexpr size_t cols_b_smem(int n2) {
  return (size_t)n2 * kPanel * (2 * sizeof(float2) + 3 * sizeof(float));
}

// Screen terms of the panel elements of this block (r = kNoPixel outside the image).
__device__ __forceinline__ void cols_b_phases(const DevPlan &p, int n1, int n2, int cg, int k1,
                                              const ScreenTable &scr, uint32_t *pa,
                                              uint32_t *pk, float *pr) {
  for (int e = threadIdx.x; e < n2 * kPanel; e += blockDim.x) {
    const int k2 = e / kPanel, col = e % kPanel;
    const int x = cg * kPanel + col;
    const int y = image_row_of(k1 + n1 * k2, p.nv, p.height);
    if (x < p.width && y >= 0) {
      const size_t i = (size_t)y * p.width + x;
      pa[e] = __ldg(scr.a + i);
      pk[e] = __ldg(scr.k + i);
      pr[e] = __ldg(scr.r + i);
    } else {
      pr[e] = kNoPixel;
    }
  }
}

// Pass B (forward) with the fused w-screen and accumulation over the batch;
// NE >= n2 * kPanel / blockDim.x accumulators per thread.
template <int NE>
__global__ void __launch_bounds__(kColThreads, 2)
    fft_cols_forward_accumulate_kernel(FftDesc d2, DevPlan p, int n1,
                                       float2 *__restrict__ R, int rstride,
                                       int n_batch, int p_begin,
                                       const ScreenTable scr,
                                       float2 *__restrict__ acc,
                                       const float2 *__restrict__ tw2,
                                       const uint8_t *__restrict__ flags) {
  extern __shared__ float2 s[];
  const int n2 = d2.L;
  const int nv = p.nv;
  const int cg = blockIdx.x, k1 = blockIdx.y;
  const int ne = n2 * kPanel;
  uint32_t *pa = reinterpret_cast<uint32_t *>(s + 2 * ne);
  uint32_t *pk = pa + ne;
  float *pr = reinterpret_cast<float *>(pk + ne);
  cols_b_phases(p, n1, n2, cg, k1, scr, pa, pk, pr);
  float part[NE];
#pragma unroll
  for (int c = 0; c < NE; ++c) part[c] = 0.f;
  for (int b = 0; b < n_batch; ++b) {
    const float2 *base = R + (size_t)b * nv * rstride + (size_t)n2 * k1 * rstride + cg * kPanel;
    // flags (set only when no pass A ran before): unflagged rows read as zeros
    load_panel(s, base, (size_t)rstride, n2,
               flags ? flags + (size_t)b * nv + (size_t)n2 * k1 : nullptr, 1);
    __syncthreads();
    const float2 *res = fft_smem<kPanelLayout>(s, s + ne, d2, -1.0f, tw2);
#pragma unroll
    for (int c = 0; c < NE; ++c) {
      const int e = threadIdx.x + c * blockDim.x;
      if (e < ne) {
        const float r = pr[e];
        if (r != kNoPixel) {
          const float2 v = res[e];
          float sn, cs;
          screen_b(pa[e], pk[e], r, p_begin + b, &sn, &cs);
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
    if (e < ne && pr[e] != kNoPixel) {
      const int k2 = e / kPanel, col = e % kPanel;
      const int x = cg * kPanel + col;
      const int y = image_row_of(k1 + n1 * k2, nv, p.height);
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

// Pass B' (backward): screened, pre-corrected image rows -> length-n2
// backward transforms -> twiddle -> R rows n2*k1 + r2.
template <int NE>
__global__ void __launch_bounds__(kColThreads, 2)
    fft_cols_backward_screen_kernel(FftDesc d2, DevPlan p, int n1,
                                    const float *__restrict__ img_corr,
                                    const ScreenTable scr,
                                    float2 *__restrict__ R, int rstride,
                                    int n_batch, int p_begin,
                                    const float2 *__restrict__ tw2,
                                    const float2 *__restrict__ twN) {
  extern __shared__ float2 s[];
  const int n2 = d2.L;
  const int nv = p.nv;
  const int cg = blockIdx.x, k1 = blockIdx.y;
  const int ne = n2 * kPanel;
  uint32_t *pa = reinterpret_cast<uint32_t *>(s + 2 * ne);
  uint32_t *pk = pa + ne;
  float *pr = reinterpret_cast<float *>(pk + ne);
  cols_b_phases(p, n1, n2, cg, k1, scr, pa, pk, pr);
  float val[NE];  // pre-corrected image value of each element
#pragma unroll
  for (int c = 0; c < NE; ++c) {
    const int e = threadIdx.x + c * blockDim.x;
    val[c] = 0.f;
    if (e < ne) {
      const int k2 = e / kPanel, col = e % kPanel;
      const int x = cg * kPanel + col;
      const int y = image_row_of(k1 + n1 * k2, nv, p.height);
      if (x < p.width && y >= 0) val[c] = __ldg(img_corr + (size_t)y * p.width + x);
    }
  }
  __syncthreads();
  for (int b = 0; b < n_batch; ++b) {
#pragma unroll
    for (int c = 0; c < NE; ++c) {
      const int e = threadIdx.x + c * blockDim.x;
      if (e < ne) {
        float2 v = make_float2(0.f, 0.f);
        if (val[c] != 0.0f) {
          float sn, cs;
          screen_b(pa[e], pk[e], pr[e], p_begin + b, &sn, &cs);
          v = make_float2(val[c] * cs, val[c] * sn);  // a exp(+2 pi i t)
        }
        s[e] = v;
      }
    }
    __syncthreads();
    const float2 *res = fft_smem<kPanelLayout>(s, s + ne, d2, +1.0f, tw2);
    float2 *base = R + (size_t)b * nv * rstride + (size_t)n2 * k1 * rstride + cg * kPanel;
    for (int e = threadIdx.x; e < ne; e += blockDim.x) {
      const int r2 = e / kPanel, c = e % kPanel;
      float2 v = res[e];
      if (n1 > 1) {
        float2 w = __ldg(twN + r2 * k1);  // r2 < n2, k1 < n1: r2 k1 < nv
        w.y = -w.y;  // exp(+2 pi i r2 k1 / nv)
        v = cmul(v, w);
      }
      base[(size_t)r2 * rstride + c] = v;
    }
    __syncthreads();
  }
}

// ---------------------------------------------- two-stage panel transforms ----
// Column transforms of length N = 16 R2 (R2 <= 8) over a panel of 32 columns,
// in two Stockham stages and one shared-memory round trip:
//   stage 1, radix 16 (p = 1): butterfly (i < R2, column b) takes panel rows
//     i + t R2 (t < 16) straight from `load` into registers and writes its
//     outputs to s[(16 i + q) * 32 + b];
//   stage 2, radix R2 (p = 16): butterfly (i < 16, b) reads s[(i + 16 t) * 32 +
//     b], twiddles by exp(sign 2 pi i t i / N), and hands output row i + 16 q
//     (natural order) to `store`.
// kPanelThreads threads: stage 1 has R2 * 32 <= 256 butterflies, stage 2 has
// 512, two per thread (slot = it * R2 + q numbers a thread's outputs).
constexpr int kPanelThreads = 256;

template <int R2, class Load, class Store>
__device__ __forceinline__ void panel_fft(float2 *__restrict__ s, float sign,
                                          const float2 *__restrict__ tw, Load load, Store store) {
  const int b = threadIdx.x & 31;
  if (threadIdx.x < R2 * 32) {
    const int i = threadIdx.x >> 5;
    float2 v[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) v[t] = load(t, i + t * R2, b);
    dft<16>(v, sign);
#pragma unroll
    for (int q = 0; q < 16; ++q) s[(16 * i + q) * 32 + b] = v[q];
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const int i = (threadIdx.x >> 5) + 8 * it;
    float2 v[R2];
#pragma unroll
    for (int t = 0; t < R2; ++t) v[t] = s[(i + 16 * t) * 32 + b];
    if (i > 0) {
#pragma unroll
      for (int t = 1; t < R2; ++t) {
        float2 w = __ldg(tw + t * i);  // exp(-2 pi i t i / N)
        w.y *= -sign;
        v[t] = cmul(v[t], w);
      }
    }
    dft<R2>(v, sign);
#pragma unroll
    for (int q = 0; q < R2; ++q) store(it * R2 + q, i + 16 * q, b, v[q]);
  }
}

// Pass A / A' with the two-stage panel transform (n1 = 16 R2): panel row e is
// row r2 + n2 e of plane blockIdx.z; forward reads unflagged rows as zeros and
// applies the four-step twiddle w_nv^(r2 k1), backward writes flagged rows only.
template <int R2>
__global__ void __launch_bounds__(kPanelThreads)
    fft_cols_pass_a16_kernel(float2 *__restrict__ R, int rstride, int nv, int n2, float sign,
                             const float2 *__restrict__ tw1, const float2 *__restrict__ twN,
                             const uint8_t *__restrict__ flags) {
  __shared__ float2 s[16 * R2 * 32];
  const int cg = blockIdx.x, r2 = blockIdx.y;
  float2 *base = R + (size_t)blockIdx.z * nv * rstride + cg * kPanel;
  const uint8_t *fl = flags ? flags + (size_t)blockIdx.z * nv : nullptr;
  const bool fwd = sign < 0;
  auto load = [&](int, int e, int c) -> float2 {
    const int row = r2 + n2 * e;
    if (fwd && fl && !__ldg(fl + row)) return make_float2(0.f, 0.f);
    return __ldg(base + (size_t)row * rstride + c);
  };
  auto store = [&](int, int k1, int c, float2 v) {
    const int row = r2 + n2 * k1;
    if (fwd) {
      v = cmul(v, __ldg(twN + r2 * k1));  // r2 k1 < nv
      base[(size_t)row * rstride + c] = v;
    } else if (!fl || __ldg(fl + row)) {
      base[(size_t)row * rstride + c] = v;
    }
  };
  panel_fft<R2>(s, sign, tw1, load, store);
}

// Shared bytes of the two-stage pass B kernels: the FFT buffer (n2 * kPanel
// float2) and the screen terms a, k, r (n2 * kPanel words each).
__host__ __device__ constexpr size_t cols_b16_smem(int n2) {
  return (size_t)n2 * kPanel * (sizeof(float2) + 3 * sizeof(float));
}

// Pass B (forward, n2 = 16 R2) with the fused w-screen: a thread's stage-2
// outputs (slot it R2 + q: row (tid >> 5) + 8 it + 16 q, column tid & 31) are
// the same for every plane, so their screened real parts sum over the batch in
// registers and go once into the image accumulator (Kahan).  flags (set only
// when no pass A ran before): unflagged rows of R read as zeros.
template <int R2>
__global__ void __launch_bounds__(kPanelThreads, 2)
    fft_cols_forward_accumulate16_kernel(DevPlan p, int n1, float2 *__restrict__ R, int rstride,
                                         int n_batch, int p_begin,
                                         const ScreenTable scr,
                                         float2 *__restrict__ acc,
                                         const float2 *__restrict__ tw2,
                                         const uint8_t *__restrict__ flags) {
  extern __shared__ float2 s[];
  constexpr int N = 16 * R2, ne = N * kPanel;
  const int nv = p.nv;
  const int cg = blockIdx.x, k1 = blockIdx.y;
  uint32_t *pa = reinterpret_cast<uint32_t *>(s + ne);
  uint32_t *pk = pa + ne;
  float *pr = reinterpret_cast<float *>(pk + ne);
  cols_b_phases(p, n1, N, cg, k1, scr, pa, pk, pr);
  float part[2 * R2];
#pragma unroll
  for (int c = 0; c < 2 * R2; ++c) part[c] = 0.f;
  for (int b = 0; b < n_batch; ++b) {
    const float2 *base = R + (size_t)b * nv * rstride + (size_t)N * k1 * rstride + cg * kPanel;
    const uint8_t *fl = flags ? flags + (size_t)b * nv + (size_t)N * k1 : nullptr;
    auto load = [&](int, int e, int c) -> float2 {
      if (fl && !__ldg(fl + e)) return make_float2(0.f, 0.f);
      return __ldg(base + (size_t)e * rstride + c);
    };
    auto store = [&](int slot, int k2, int c, float2 v) {
      const int e = k2 * kPanel + c;
      const float r = pr[e];
      if (r != kNoPixel) {
        float sn, cs;
        screen_b(pa[e], pk[e], r, p_begin + b, &sn, &cs);
        // Re(v exp(-2 pi i t)) = v.re cos + v.im sin
        part[slot] += v.x * cs + v.y * sn;
      }
    };
    panel_fft<R2>(s, -1.0f, tw2, load, store);
    __syncthreads();  // the next plane's stage 1 rewrites s
  }
  const int col = threadIdx.x & 31;
#pragma unroll
  for (int it = 0; it < 2; ++it) {
#pragma unroll
    for (int q = 0; q < R2; ++q) {
      const int k2 = (threadIdx.x >> 5) + 8 * it + 16 * q;
      const int e = k2 * kPanel + col;
      if (pr[e] != kNoPixel) {
        const int x = cg * kPanel + col;
        const int y = image_row_of(k1 + n1 * k2, nv, p.height);
        float2 *a = acc + (size_t)y * p.width + x;
        float2 sc = *a;  // (sum, compensation)
        const float yv = part[it * R2 + q] - sc.y;
        const float t = sc.x + yv;
        sc.y = (t - sc.x) - yv;
        sc.x = t;
        *a = sc;
      }
    }
  }
}

// Pass B' (backward, n2 = 16 R2): screened, pre-corrected image rows -> length
// n2 backward transforms -> twiddle -> R rows n2 k1 + r2.  A stage-1 thread
// keeps the 16 image values it feeds (rows i + t R2 of its column).
template <int R2>
__global__ void __launch_bounds__(kPanelThreads, 2)
    fft_cols_backward_screen16_kernel(DevPlan p, int n1, const float *__restrict__ img_corr,
                                      const ScreenTable scr, float2 *__restrict__ R,
                                      int rstride, int n_batch, int p_begin,
                                      const float2 *__restrict__ tw2,
                                      const float2 *__restrict__ twN) {
  extern __shared__ float2 s[];
  constexpr int N = 16 * R2, ne = N * kPanel;
  const int nv = p.nv;
  const int cg = blockIdx.x, k1 = blockIdx.y;
  uint32_t *pa = reinterpret_cast<uint32_t *>(s + ne);
  uint32_t *pk = pa + ne;
  float *pr = reinterpret_cast<float *>(pk + ne);
  cols_b_phases(p, n1, N, cg, k1, scr, pa, pk, pr);
  const int col = threadIdx.x & 31, i1 = threadIdx.x >> 5;
  float val[16];
#pragma unroll
  for (int t = 0; t < 16; ++t) {
    val[t] = 0.f;
    if (i1 < R2) {
      const int x = cg * kPanel + col;
      const int y = image_row_of(k1 + n1 * (i1 + t * R2), nv, p.height);
      if (x < p.width && y >= 0) val[t] = __ldg(img_corr + (size_t)y * p.width + x);
    }
  }
  __syncthreads();  // screen terms
  for (int b = 0; b < n_batch; ++b) {
    float2 *base = R + (size_t)b * nv * rstride + (size_t)N * k1 * rstride + cg * kPanel;
    auto load = [&](int t, int e, int c) -> float2 {
      if (val[t] == 0.0f) return make_float2(0.f, 0.f);
      const int idx = e * kPanel + c;
      float sn, cs;
      screen_b(pa[idx], pk[idx], pr[idx], p_begin + b, &sn, &cs);
      return make_float2(val[t] * cs, val[t] * sn);  // a exp(+2 pi i t)
    };
    auto store = [&](int, int r2, int c, float2 v) {
      if (n1 > 1) {
        float2 w = __ldg(twN + r2 * k1);  // r2 < n2, k1 < n1: r2 k1 < nv
        w.y = -w.y;                        // exp(+2 pi i r2 k1 / nv)
        v = cmul(v, w);
      }
      base[(size_t)r2 * rstride + c] = v;
    };
    panel_fft<R2>(s, +1.0f, tw2, load, store);
    __syncthreads();
  }
}

void set_smem(const void *fn, size_t bytes) { ensure_dynamic_smem(fn, bytes); }

}  // namespace

// Per-stage twiddle tables of the row schedule of length L (cached).
static const float2 *row_stage_twiddles(FftTables &t, const FftDesc &d, RowStages *st) {
  std::lock_guard<std::mutex> lock(t.mu);
  int p = 1, off = 0;
  for (int s = 0; s < d.n_stages; ++s) {
    st->tw_off[s] = off;
    off += p * (d.radix[s] - 1);
    p *= d.radix[s];
  }
  auto it = t.row_tables.find(d.L);
  if (it != t.row_tables.end()) return it->second;
  std::vector<float2> h((size_t)std::max(off, 1));
  p = 1;
  for (int s = 0; s < d.n_stages; ++s) {
    const int R = d.radix[s];
    for (int tt = 1; tt < R; ++tt)
      for (int k = 0; k < p; ++k) {
        // exp(-2 pi i t k / (p R)), argument reduced exactly in FP64
        const long long num = (long long)tt * k % ((long long)p * R);
        const double a = -2.0 * M_PI * (double)num / ((double)p * R);
        h[st->tw_off[s] + (tt - 1) * p + k] = make_float2((float)std::cos(a), (float)std::sin(a));
      }
    p *= R;
  }
  float2 *dd = nullptr;
  WGPU_CUDA(cudaMalloc(&dd, sizeof(float2) * h.size()));
  WGPU_CUDA(cudaMemcpy(dd, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice));
  t.row_tables[d.L] = dd;
  return dd;
}

// Row lengths the persistent kernel handles (radix 16, radix-16 stages, an
// optional radix-8 stage, one last stage of radix 2, 3 or 5).
static bool persistent_schedule(const FftDesc &d, int *last, bool *mid8) {
  if (d.n_stages < 2 || d.radix[0] != 16) return false;
  *last = d.radix[d.n_stages - 1];
  *mid8 = false;
  for (int s = 1; s + 1 < d.n_stages; ++s) {
    if (d.radix[s] == 16 && !*mid8) continue;
    if (d.radix[s] == 8 && s + 2 == d.n_stages) { *mid8 = true; continue; }
    return false;
  }
  return (*last == 2 && !*mid8) || (*last == 3 && !*mid8) || (*last == 5 && *mid8);
}

bool fft_row_length_supported(int L) {
  if (L % 16 || L > kFftMaxRow) return false;
  if (L <= kRowPingPongMax) return true;
  FftDesc d;
  try {
    d = make_desc(L, true);
  } catch (const Error &) {
    return false;
  }
  int last;
  bool mid8;
  return persistent_schedule(d, &last, &mid8);
}

void fft_prepare_rows(FftTables &t, int L) {
  RowStages st;
  row_stage_twiddles(t, make_desc(L, true), &st);
}

template <bool FWD, int LAST, bool MID8>
static void launch_persistent(const FftDesc &d, const RowStages &st, const float2 *tws,
                              const DevPlan &p, const float2 *in, int in_stride, float2 *out,
                              int out_stride, int n_batch, const RowSel &sel, unsigned *err,
                              cudaStream_t s) {
  const int n_rows = n_batch * p.nv;
  const int buf_elems = std::max(p.nu, in_stride);
  const uint32_t in_bytes = (uint32_t)(sizeof(float2) * (FWD ? p.nu : in_stride));
  if ((in_bytes & 15) || (buf_elems & 1))
    throw Error(WGPU_ERR_INVALID, "row transform sizes must be multiples of 16 bytes");
  const int threads = std::min(kRowThreadsMax, (p.nu / 16 + 31) / 32 * 32);
  size_t smem = 128 + 2 * sizeof(float2) * (size_t)buf_elems;
  // middle-stage twiddles (stages 1 .. n-2) into shared memory when they fit
  int mid_tab = d.n_stages > 2 ? st.tw_off[d.n_stages - 1] - st.tw_off[1] : 0;
  int dev = 0, smem_max = 0;
  WGPU_CUDA(cudaGetDevice(&dev));
  WGPU_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (smem + sizeof(float2) * (size_t)mid_tab <= (size_t)smem_max)
    smem += sizeof(float2) * (size_t)mid_tab;
  else
    mid_tab = 0;
  auto kern = fft_rows_persistent_kernel<FWD, LAST, MID8>;
  set_smem((const void *)kern, smem);
  int per_sm = 0;
  WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
  if (per_sm < 1) throw Error(WGPU_ERR_INVALID, "row transform does not fit on an SM");
  const int blocks = std::min(n_rows, sm_count() * per_sm);
  kern<<<blocks, threads, smem, s>>>(d, st, tws, in, in_stride, in_bytes, out, out_stride,
                                      n_batch, p.nv, sel, p.width, buf_elems, mid_tab, err);
  check_launch(FWD ? "fft_rows_persistent_kernel<forward>"
                   : "fft_rows_persistent_kernel<backward>");
}

template <bool FWD>
static void launch_rows(FftTables &t, const DevPlan &p, const float2 *in, int in_stride,
                        float2 *out, int out_stride, int n_batch, const RowSel &sel,
                        unsigned *err, cudaStream_t s) {
  const int n_rows = n_batch * p.nv;
  if (n_rows <= 0) return;
  if (p.nu % 16 || p.nu > kFftMaxRow)
    throw Error(WGPU_ERR_INVALID, "row transform length must be a multiple of 16 up to 12288");
  const FftDesc d = make_desc(p.nu, true);
  RowStages st;
  const float2 *tws = row_stage_twiddles(t, d, &st);
  if (p.nu > kRowPingPongMax) {
    int last;
    bool mid8;
    if (!persistent_schedule(d, &last, &mid8))
      throw Error(WGPU_ERR_INVALID, "row length " + std::to_string(p.nu) +
                                        " has no row transform schedule");
    if (last == 2)
      launch_persistent<FWD, 2, false>(d, st, tws, p, in, in_stride, out, out_stride, n_batch, sel,
                                       err, s);
    else if (last == 3)
      launch_persistent<FWD, 3, false>(d, st, tws, p, in, in_stride, out, out_stride, n_batch, sel,
                                       err, s);
    else
      launch_persistent<FWD, 5, true>(d, st, tws, p, in, in_stride, out, out_stride, n_batch, sel,
                                       err, s);
    return;
  }
  const int threads = std::min(kRowPingPongThreads, std::max(64, (p.nu / 16 + 31) / 32 * 32));
  const size_t smem = 2 * sizeof(float2) * (size_t)row_buffer(p.nu);
  set_smem((const void *)fft_rows_pingpong_kernel<FWD>, smem);
  fft_rows_pingpong_kernel<FWD><<<(unsigned)n_rows, threads, smem, s>>>(
      d, st, tws, in, in_stride, out, out_stride, n_batch, p.nv, sel, p.width);
  check_launch(FWD ? "fft_rows_pingpong_kernel<forward>" : "fft_rows_pingpong_kernel<backward>");
}

void launch_fft_rows_forward_crop(FftTables &t, const DevPlan &p,
                                  const float2 *planes, float2 *R, int rstride,
                                  int n_batch, const RowSel &sel, unsigned *err,
                                  cudaStream_t s) {
  launch_rows<true>(t, p, planes, p.nu, R, rstride, n_batch, sel, err, s);
}

void launch_fft_rows_backward_pad(FftTables &t, const DevPlan &p,
                                  const float2 *R, int rstride, float2 *planes,
                                  int n_batch, const RowSel &sel, unsigned *err,
                                  cudaStream_t s) {
  launch_rows<false>(t, p, R, rstride, planes, p.nu, n_batch, sel, err, s);
}

// R2 of the two-stage panel transform of length n, or 0 when n is not 16 R2
// for R2 in {2, 3, 4, 5, 6, 8} (other lengths use the generic Stockham panel
// kernels).
static int panel_r2(int n) {
  const int r = n % 16 == 0 ? n / 16 : 0;
  return (r >= 2 && r <= 8 && r != 7) ? r : 0;  // radices with a butterfly: 2, 3, 4, 5, 6, 8
}

#define WGPU_PANEL_SWITCH(r2, CALL) \
  switch (r2) {                     \
    case 2: CALL(2); break;         \
    case 3: CALL(3); break;         \
    case 4: CALL(4); break;         \
    case 5: CALL(5); break;         \
    case 6: CALL(6); break;         \
    default: CALL(8); break;        \
  }

void launch_fft_cols_a(FftTables &t, const DevPlan &p, int n1, int n2, float2 *R,
                       int rstride, int n_batch, float sign, const RowSel &sel,
                       cudaStream_t s) {
  if (n1 <= 1) return;
  const int ncg = rstride / kPanel;
  if (const int r2p = panel_r2(n1)) {
    dim3 grid(ncg, n2, n_batch);
    const float2 *tw1 = fft_twiddles(t, n1), *twN = fft_twiddles(t, p.nv);
#define WGPU_PASS_A16(X)                                                                     \
  fft_cols_pass_a16_kernel<X><<<grid, kPanelThreads, 0, s>>>(R, rstride, p.nv, n2, sign, tw1, \
                                                             twN, sel.flags)
    WGPU_PANEL_SWITCH(r2p, WGPU_PASS_A16)
#undef WGPU_PASS_A16
    check_launch("fft_cols_pass_a16_kernel");
    return;
  }
  const FftDesc d1 = make_desc(n1);
  const size_t smem = 2 * sizeof(float2) * n1 * kPanel;
  set_smem((const void *)fft_cols_pass_a_kernel, smem);
  dim3 grid(ncg, n2, n_batch);
  fft_cols_pass_a_kernel<<<grid, kColThreads, smem, s>>>(
      d1, R, rstride, p.nv, n2, sign, fft_twiddles(t, n1), fft_twiddles(t, p.nv), sel.flags);
  check_launch("fft_cols_pass_a_kernel");
}

void launch_fft_cols_b_forward_accumulate(FftTables &t, const DevPlan &p, int n1,
                                          int n2, float2 *R, int rstride,
                                          int n_batch, int p_begin,
                                          const ScreenTable &scr, float2 *acc,
                                          const RowSel &sel, cudaStream_t s) {
  // after a pass A every row of R holds data; without one, R is as the row
  // transforms left it
  const uint8_t *flags = n1 <= 1 ? sel.flags : nullptr;
  const int ncg = rstride / kPanel;
  if (const int r2p = panel_r2(n2)) {
    dim3 grid(ncg, n1);
    const float2 *tw = fft_twiddles(t, n2);
    const size_t smem = cols_b16_smem(n2);
#define WGPU_PASS_B16(X)                                                                  \
  set_smem((const void *)fft_cols_forward_accumulate16_kernel<X>, smem);                  \
  fft_cols_forward_accumulate16_kernel<X><<<grid, kPanelThreads, smem, s>>>(              \
      p, n1, R, rstride, n_batch, p_begin, scr, acc, tw, flags)
    WGPU_PANEL_SWITCH(r2p, WGPU_PASS_B16)
#undef WGPU_PASS_B16
    check_launch("fft_cols_forward_accumulate16_kernel");
    return;
  }
  const FftDesc d2 = make_desc(n2);
  const size_t smem = cols_b_smem(n2);
  dim3 grid(ncg, n1);
  const float2 *tw = fft_twiddles(t, n2);
  if (n2 * kPanel <= 8 * kColThreads) {
    set_smem((const void *)fft_cols_forward_accumulate_kernel<8>, smem);
    fft_cols_forward_accumulate_kernel<8><<<grid, kColThreads, smem, s>>>(
        d2, p, n1, R, rstride, n_batch, p_begin, scr, acc, tw, flags);
  } else {
    set_smem((const void *)fft_cols_forward_accumulate_kernel<16>, smem);
    fft_cols_forward_accumulate_kernel<16><<<grid, kColThreads, smem, s>>>(
        d2, p, n1, R, rstride, n_batch, p_begin, scr, acc, tw, flags);
  }
  check_launch("fft_cols_forward_accumulate_kernel");
}

void launch_fft_cols_b_backward_screen(FftTables &t, const DevPlan &p, int n1,
                                       int n2, const float *img_corr,
                                       const ScreenTable &scr, float2 *R,
                                       int rstride, int n_batch, int p_begin,
                                       cudaStream_t s) {
  const int ncg = rstride / kPanel;
  if (const int r2p = panel_r2(n2)) {
    dim3 grid(ncg, n1);
    const float2 *tw = fft_twiddles(t, n2), *twN = fft_twiddles(t, p.nv);
    const size_t smem = cols_b16_smem(n2);
#define WGPU_PASS_B16B(X)                                                                 \
  set_smem((const void *)fft_cols_backward_screen16_kernel<X>, smem);                     \
  fft_cols_backward_screen16_kernel<X><<<grid, kPanelThreads, smem, s>>>(                 \
      p, n1, img_corr, scr, R, rstride, n_batch, p_begin, tw, twN)
    WGPU_PANEL_SWITCH(r2p, WGPU_PASS_B16B)
#undef WGPU_PASS_B16B
    check_launch("fft_cols_backward_screen16_kernel");
    return;
  }
  const FftDesc d2 = make_desc(n2);
  const size_t smem = cols_b_smem(n2);
  dim3 grid(ncg, n1);
  const float2 *tw = fft_twiddles(t, n2), *twN = fft_twiddles(t, p.nv);
  if (n2 * kPanel <= 8 * kColThreads) {
    set_smem((const void *)fft_cols_backward_screen_kernel<8>, smem);
    fft_cols_backward_screen_kernel<8><<<grid, kColThreads, smem, s>>>(
        d2, p, n1, img_corr, scr, R, rstride, n_batch, p_begin, tw, twN);
  } else {
    set_smem((const void *)fft_cols_backward_screen_kernel<16>, smem);
    fft_cols_backward_screen_kernel<16><<<grid, kColThreads, smem, s>>>(
        d2, p, n1, img_corr, scr, R, rstride, n_batch, p_begin, tw, twN);
  }
  check_launch("fft_cols_backward_screen_kernel");
}

// Runs the bounded-wait self-test on the current device; returns
// WGPU_ERR_TIMEOUT when the wait expired and reported it (the expected
// outcome), WGPU_OK if it did not.
int bounded_wait_selftest(double timeout_ms) {
  int dev = 0, khz = 0;
  WGPU_CUDA(cudaGetDevice(&dev));
  WGPU_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev));
  const long long cycles = (long long)(timeout_ms * (double)khz);
  unsigned *d_err = nullptr, h_err = 0;
  WGPU_CUDA(cudaMalloc(&d_err, sizeof(unsigned)));
  cudaError_t e = cudaMemset(d_err, 0, sizeof(unsigned));
  if (e == cudaSuccess) {
    bounded_wait_selftest_kernel<<<1, 64>>>(cycles, d_err);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&h_err, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost);
  cudaFree(d_err);
  if (e != cudaSuccess) throw Error(WGPU_ERR_CUDA, cudaGetErrorString(e));
  count_launch();
  return h_err ? WGPU_ERR_TIMEOUT : WGPU_OK;
}

}  // namespace wgpu
