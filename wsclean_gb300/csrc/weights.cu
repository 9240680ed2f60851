// Imaging weights and the per-row weighting of raw measurement-set rows on the
// device.
//
// The weight grid follows ImageWeights (structures/imageweights.h,
// structures/imageweights.cpp): a width x height/2 half-plane of doubles into
// which every sample's visibility weights are summed (Grid), turned into
// natural, uniform or Briggs weights (FinishGridding), optionally tapered, and
// sampled per (u, v) (GetWeight).  The row preparation follows
// MsGridderData::CalculateWeightsImplementation, ApplyWeights and CollapseData
// (gridding/msgridderdata.h:36-52, 760-886): PSF point-source visibilities,
// model subtraction, selection, the visibility weighting mode, the imaging
// weight, the weighted sums and the collapse to one value per sample.
//
// Cell indices and every grid value that the host computes with a product
// followed by a sum are formed here with one rounding per operation
// (__dmul_rn / __dadd_rn), so that a sample falls into the same cell, and a
// taper compares against the same distance, as with separately rounded
// host arithmetic.
#include <cmath>
#include <cstring>
#include <string>

#include "polarization.cuh"
#include "wgpu_internal.h"

struct wgpu_imageweights {
  int mode = WGPU_WEIGHT_UNIFORM;
  double robustness = 0.0;
  int64_t width = 0, height = 0;  // after the super weight, both even
  double psx = 0.0, psy = 0.0;
  bool as_taper = false;
  bool finished = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  double *grid = nullptr;      // width * height / 2
  float *gridf = nullptr;      // (float)grid, refreshed before the rows are weighted
  bool gridf_dirty = true;
  double *sums = nullptr;      // [0] gridded weight sum, [1] sum of squares
  double *partials = nullptr;  // per-block partial sums of the reductions
  static constexpr int kScratch = 10;
  void *scratch[kScratch] = {};
  size_t scratch_bytes[kScratch] = {};
};

namespace wgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kReduceBlocks = 1024;  // fixed, so reductions add in a fixed order

unsigned blocks_for(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// Per-channel constants of the cell computation (chan_scale_kernel).
struct ChanScale {
  double lambda;
  float su, sv;
};

// uvToXY and isWithinLimits (imageweights.h:74-96): reflect into v >= 0,
// x = floor(u * W * psx + W / 2), y = floor(v * H * psy), inside when
// 0 <= x < W and y < H / 2.  Returns the cell index or -1.
__device__ __forceinline__ int64_t uv_cell(double u, double v, int64_t W, int64_t H, double psx,
                                           double psy) {
  if (v < 0.0) {
    u = -u;
    v = -v;
  }
  const double fx = floor(__dadd_rn(__dmul_rn(__dmul_rn(u, (double)W), psx), (double)(W / 2)));
  const double fy = floor(__dmul_rn(__dmul_rn(v, (double)H), psy));
  if (!(fx >= 0.0 && fx < (double)W && fy >= 0.0 && fy < (double)(H / 2))) return -1;
  return (int64_t)fx + (int64_t)fy * W;
}

// xyToUV (imageweights.h:83-91) for a cell of the half-plane.
__device__ __forceinline__ void cell_uv(int64_t x, int64_t y, int64_t W, int64_t H, double psx,
                                        double psy, double *u, double *v) {
  *u = (double)(x - W / 2) / __dmul_rn((double)W, psx);
  *v = (double)y / __dmul_rn((double)H, psy);
}

__device__ __forceinline__ double dist_sq(double u, double v) {
  return __dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v));
}

// tukeyFrom0ToN (imageweights.h:114-116): 0 at x = 0, 1 at x = n.
__device__ __forceinline__ double tukey(double x, double n) {
  return __dmul_rn(0.5, __dadd_rn(1.0, cos(__dmul_rn(M_PI / n, x - n))));
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of one value per thread over the block (kThreads threads), result in
// thread 0, added in a fixed order.
__device__ double block_sum(double v) {
  __shared__ double part[kThreads / 32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) part[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < kThreads / 32; ++k) t += part[k];
  __syncthreads();
  return t;
}

// Per-channel constants: the wavelength as the host forms it (c / f in
// double) and the FP32 scales W psx / lambda and H psy / lambda of the cell
// estimate.
__global__ void chan_scale_kernel(const double *freq, int64_t n_chan, int64_t W, int64_t H,
                                  double psx, double psy, ChanScale *t) {
  const int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ch >= n_chan) return;
  const double lambda = kSpeedOfLight / freq[ch];
  ChanScale c;
  c.lambda = lambda;
  c.su = (float)(((double)W * psx) / lambda);
  c.sv = (float)(((double)H * psy) / lambda);
  t[ch] = c;
}

// Conversions between float and double done with integer operations on the
// bit patterns: this GPU's FP64 pipe (which also executes F2F conversions and
// double compares) is a small fraction of its FP32 rate, and the per-sample
// paths below use none of it.
//
// float -> double, exact (zeros, subnormals, infinities and NaNs included).
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  unsigned long long r;
  if (e == 0xffu) {
    r = 0x7ff0000000000000ull | ((unsigned long long)m << 29);
  } else if (e != 0u) {
    r = ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
  } else if (m == 0u) {
    r = 0ull;
  } else {  // subnormal m * 2^-149 with its top bit at position p
    const int p = 31 - __clz((int)m);
    r = ((unsigned long long)(p + 874) << 52) |
        (((unsigned long long)m << (52 - p)) & 0xfffffffffffffull);
  }
  return __longlong_as_double((long long)(sign | r));
}

// double -> float by truncating the mantissa (error below one float ulp);
// magnitudes under 2^-126 become zero; false when beyond the float range,
// infinite or NaN.
__device__ __forceinline__ bool d2f_trunc(unsigned long long b, float *out) {
  const unsigned hi = (unsigned)(b >> 32);
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  const unsigned sign = hi & 0x80000000u;
  if (e >= 255) return false;
  if (e <= 0) {
    *out = __uint_as_float(sign);
    return true;
  }
  *out = __uint_as_float(sign | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7fffffu));
  return true;
}

// The cell of (um, vm) metres at one channel, decided in FP32.  The FP32
// estimate x' = um * su + W/2 (um truncated to float: < 1 ulp; su and the
// fused multiply-add rounded: 1/2 ulp each) differs from the host's double
// evaluation (u = um / lambda, then u * W * psx + W / 2, each rounded) by less
// than 2^-22 (|um su| + |x'|); y' = vm * sv by less than 2^-22 |y'|.  A cell
// is decided when both coordinates lie farther than twice (x) or four times
// (y) that from a cell edge.  Returns the cell, -1 when decided outside the
// grid, -2 when undecided (also for non-finite inputs, |vm| below 2^-930,
// whose sign the division by the wavelength could lose, and values beyond the
// float range).  Reflection into v >= 0 flips the signs exactly.
__device__ __forceinline__ int64_t fast_cell(double um, double vm, const ChanScale &c, int64_t W,
                                             int64_t H) {
  // grid sizes are below 2^21: 32-bit integer <-> float conversions (the
  // 64-bit ones also run on the FP64 pipe)
  const int w32 = (int)W, hh32 = (int)(H / 2);
  const unsigned long long bu = (unsigned long long)__double_as_longlong(um);
  const unsigned long long bv = (unsigned long long)__double_as_longlong(vm);
  const unsigned long long av = bv & 0x7fffffffffffffffull;
  if (!(av == 0ull || (av >= 0x05d0000000000000ull && av <= 0x7ff0000000000000ull))) return -2;
  const unsigned long long flip = (bv >> 63 != 0ull && av != 0ull) ? (1ull << 63) : 0ull;
  float uf, vf;
  if (!d2f_trunc(bu ^ flip, &uf) || !d2f_trunc(av, &vf)) return -2;
  const float xf = fmaf(uf, c.su, (float)(w32 / 2));
  const float bx = 0x1p-21f * (fabsf(uf * c.su) + fabsf(xf)) + 1e-30f;
  const float kx = floorf(xf), fx = xf - kx;
  if (!(fx > bx && fx < 1.0f - bx)) return -2;
  const float yf = vf * c.sv;
  const float by = 0x1p-20f * fabsf(yf) + 1e-30f;
  const float ky = floorf(yf), fy = yf - ky;
  if (!(fy > by && fy < 1.0f - by)) return -2;
  if (!(kx >= 0.0f && kx < (float)w32 && ky >= 0.0f && ky < (float)hh32)) return -1;
  return (int64_t)(int)kx + (int64_t)(int)ky * (int64_t)w32;
}

// Float-float accumulator (Knuth's TwoSum), flushed into a double every
// kFlush additions: sums of float weights in the FP32 pipe with a relative
// error far below that of the reference's own serial double sum.
struct FloatSum {
  double acc = 0.0;
  float hi = 0.0f, lo = 0.0f;
  int n = 0;
  static constexpr int kFlush = 32;
  __device__ __forceinline__ void add(float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
    if (++n == kFlush) flush();
  }
  __device__ __forceinline__ void flush() {
    acc += f2d_bits(hi) + f2d_bits(lo);
    hi = lo = 0.0f;
    n = 0;
  }
  __device__ __forceinline__ double value() {
    flush();
    return acc;
  }
};

// Undecided samples of one pass: block b appends to its own slice
// [b * cap, (b + 1) * cap) of the list (cap = the samples a block visits),
// counting in shared memory; counts[b] holds the slice's length afterwards.
struct Pending {
  uint32_t *idx;
  uint32_t *counts;
  uint32_t cap;
};

__device__ __forceinline__ void pending_push(const Pending &p, uint32_t *s_count, bool want,
                                             uint32_t e) {
  const unsigned m = __ballot_sync(0xffffffffu, want);
  if (m == 0) return;
  const int lane = threadIdx.x & 31;
  uint32_t base = 0;
  if (lane == __ffs(m) - 1) base = atomicAdd(s_count, (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
  if (want) p.idx[(size_t)blockIdx.x * p.cap + base + __popc(m & ((1u << lane) - 1))] = e;
}

// Adds one sample's correlation weights (1 for a non-zero weight when the
// weights are a taper) to its cell: their float-float sum (hi, lo) goes to
// the cell as one or two double atomic adds, which L2 performs.
__device__ __forceinline__ void grid_sample(double *cellp, const float *w, int n_pol,
                                            int as_taper, FloatSum &tot) {
  float hi = 0.0f, lo = 0.0f;
  for (int p = 0; p < n_pol; ++p) {
    float x = w[p];
    if (as_taper && x != 0.0f) x = 1.0f;
    const float sum = hi + x;
    const float bp = sum - hi;
    lo += (hi - (sum - bp)) + (x - bp);
    hi = sum;
  }
  if (hi != 0.0f) {
    atomicAdd(cellp, f2d_bits(hi));
    tot.add(hi);
  }
  if (lo != 0.0f) {
    atomicAdd(cellp, f2d_bits(lo));
    tot.add(lo);
  }
}

// Grid(MSProvider &, BandData) (imageweights.cpp:75-112), first pass, over a
// fixed grid of blocks: for every (row, channel) with an FP32-decided cell the
// correlations' weights (1 for a non-zero weight when the weights are a
// taper) are summed and added to the cell; undecided samples go to the
// pending list.  The row's (u, v) reflection into v >= 0 happens in metres,
// as in the reference.
__global__ void __launch_bounds__(kThreads) weight_grid_fast_kernel(
    double *grid, double *total, int64_t W, int64_t H, int as_taper, uint32_t n,
    uint32_t n_chan, int n_pol, const double *uvw, const ChanScale *cs, const float *weights,
    Pending pend) {
  __shared__ uint32_t s_count;
  if (threadIdx.x == 0) s_count = 0;
  __syncthreads();
  FloatSum tot;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t e = base + threadIdx.x;
    bool undecided = false;
    if (e < n) {
      const uint32_t r = e / n_chan, ch = e - r * n_chan;
      const int64_t cell = fast_cell(uvw[3 * (size_t)r], uvw[3 * (size_t)r + 1], cs[ch], W, H);
      undecided = cell == -2;
      if (cell >= 0) grid_sample(grid + cell, weights + (size_t)e * n_pol, n_pol, as_taper, tot);
    }
    pending_push(pend, &s_count, undecided, e);
  }
  const double t = block_sum(tot.value());
  if (threadIdx.x == 0) {
    pend.counts[blockIdx.x] = s_count;
    if (t != 0.0) atomicAdd(total, t);
  }
}

// Second pass over the pending samples: the cell as the host computes it, in
// double (reflection in metres, u = um / lambda, v = vm / lambda).
__global__ void __launch_bounds__(kThreads) weight_grid_exact_kernel(
    double *grid, double *total, int64_t W, int64_t H, double psx, double psy, int as_taper,
    uint32_t n_chan, int n_pol, const double *uvw, const ChanScale *cs, const float *weights,
    Pending pend) {
  const uint32_t count = pend.counts[blockIdx.x];
  const uint32_t *list = pend.idx + (size_t)blockIdx.x * pend.cap;
  FloatSum tot;
  for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
    const uint32_t e = list[i];
    const uint32_t r = e / n_chan, ch = e - r * n_chan;
    double um = uvw[3 * (size_t)r], vm = uvw[3 * (size_t)r + 1];
    if (vm < 0.0) {
      um = -um;
      vm = -vm;
    }
    const double lambda = cs[ch].lambda;
    const int64_t cell = uv_cell(um / lambda, vm / lambda, W, H, psx, psy);
    if (cell >= 0) grid_sample(grid + cell, weights + (size_t)e * n_pol, n_pol, as_taper, tot);
  }
  const double t = block_sum(tot.value());
  if (threadIdx.x == 0 && t != 0.0) atomicAdd(total, t);
}

// Partial sums of grid^2 over a fixed grid of kReduceBlocks blocks.
__global__ void sum_sq_partials_kernel(const double *grid, int64_t n, double *partials) {
  double local = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    local += grid[i] * grid[i];
  const double t = block_sum(local);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

__global__ void sum_partials_kernel(const double *partials, int n, double *out) {
  double local = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) local += partials[i];
  const double t = block_sum(local);
  if (threadIdx.x == 0) *out = t;
}

// FinishGridding (imageweights.cpp:114-147): cells without coverage stay 0.
__global__ void weight_finish_kernel(double *grid, int64_t n, int mode, double s_sq) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double val = grid[i];
  if (val == 0.0) return;
  if (mode == WGPU_WEIGHT_BRIGGS)
    grid[i] = 1.0 / __dadd_rn(1.0, __dmul_rn(val, s_sq));
  else if (mode == WGPU_WEIGHT_UNIFORM)
    grid[i] = 1.0 / val;
  else
    grid[i] = 1.0;
}

// The uv-range limits and tapers of imageweights.cpp:149-282 and 328-351, one
// thread per cell.  a, b as documented for WGPU_TAPER_*; for the Gaussian
// taper a is the host-computed -2 sigma^2 term.
__global__ void weight_taper_kernel(double *grid, int64_t W, int64_t H, double psx, double psy,
                                    int kind, double a, double b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W * (H / 2)) return;
  const int64_t y = i / W, x = i - y * W;
  double u, v;
  cell_uv(x, y, W, H, psx, psy, &u, &v);
  double g = grid[i];
  switch (kind) {
    case WGPU_TAPER_MIN_UV:
      if (dist_sq(u, v) < __dmul_rn(a, a)) g = 0.0;
      break;
    case WGPU_TAPER_MAX_UV:
      if (dist_sq(u, v) > __dmul_rn(a, a)) g = 0.0;
      break;
    case WGPU_TAPER_TUKEY: {  // a = transition, b = max uv
      const double d2 = dist_sq(u, v), max_sq = __dmul_rn(b, b), t = b - a;
      if (d2 > max_sq)
        g = 0.0;
      else if (d2 > __dmul_rn(t, t))
        g *= tukey(b - sqrt(d2), a);
      break;
    }
    case WGPU_TAPER_TUKEY_INNER: {  // a = transition, b = min uv
      const double d2 = dist_sq(u, v), min_sq = __dmul_rn(b, b), t = b + a;
      if (d2 < min_sq)
        g = 0.0;
      else if (d2 < __dmul_rn(t, t))
        g *= tukey(sqrt(d2) - b, a);
      break;
    }
    case WGPU_TAPER_EDGE:
    case WGPU_TAPER_EDGE_TUKEY: {
      double max_u, max_v;
      cell_uv(W, H / 2, W, H, psx, psy, &max_u, &max_v);
      const double ud = max_u - fabs(u), vd = max_v - fabs(v);
      if (kind == WGPU_TAPER_EDGE) {
        if (ud < a || vd < a) g = 0.0;
      } else {  // a = transition, b = edge size
        const double total = a + b;
        if (ud < b || vd < b) {
          g = 0.0;
        } else if (ud < total || vd < total) {
          double ru = ud - b, rv = vd - b;
          if (ru > a) ru = a;
          if (rv > a) rv = a;
          g *= tukey(ru, a) * tukey(rv, a);
        }
      }
      break;
    }
    case WGPU_TAPER_GAUSSIAN:
      if (g != 0.0) g = g * exp(dist_sq(u, v) / a);
      break;
    default:
      break;
  }
  grid[i] = g;
}

// RankFilter (imageweights.cpp:310-326) with windowMean (:353-388): each
// covered cell above rank_limit times the mean of the covered cells in its
// window is clipped to that value.  src is a copy of the grid; the window is
// summed in the host loop's order.
__global__ void rank_filter_kernel(const double *src, double *grid, int64_t W, int64_t Hh,
                                   double rank_limit, int64_t window) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W * Hh) return;
  const int64_t y = i / W, x = i - y * W;
  const double w = src[i];
  if (w == 0.0) return;
  const int64_t d = window / 2;
  const int64_t x1 = x <= d ? 0 : x - d, y1 = y <= d ? 0 : y - d;
  const int64_t x2 = x + d >= W ? W : x + d, y2 = y + d >= Hh ? Hh : y + d;
  int64_t count = 0;
  double sum = 0.0;
  for (int64_t yi = y1; yi < y2; ++yi)
    for (int64_t xi = x1; xi < x2; ++xi) {
      const double c = src[yi * W + xi];
      if (c != 0.0) {
        ++count;
        sum += c;
      }
    }
  const double limit = sum / (double)count * rank_limit;
  if (w > limit) grid[i] = limit;
}

__global__ void weight_fill_kernel(double *grid, int64_t n, double value) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) grid[i] = value;
}

// GetGrid (imageweights.cpp:284-300): the half-plane mirrored into a
// width x height image, row y of the grid at rows H/2 + y (as is) and
// H/2 - 1 - y (x reversed).
__global__ void weight_mirror_kernel(const double *grid, int64_t W, int64_t H, double *image) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W * (H / 2)) return;
  const int64_t y = i / W, x = i - y * W;
  const double g = grid[i];
  image[(H / 2 - 1 - y) * W + (W - x - 1)] = g;
  image[(H / 2 + y) * W + x] = g;
}

__global__ void weight_sample_kernel(const double *grid, int64_t W, int64_t H, double psx,
                                     double psy, int64_t n, const double *u, const double *v,
                                     double *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t cell = uv_cell(u[i], v[i], W, H, psx, psy);
  out[i] = cell >= 0 ? grid[cell] : 0.0;
}

// CalculateWeightsImplementation + ApplyWeights + CollapseData
// (msgridderdata.h:36-52, 760-789, 826-886) for one (row, channel) sample:
//   1. PSF mode: every correlation is 1, rotated by the phase of a point
//      source at (dl, dm) when that is not the phase centre (RotateVisibilities,
//      msgridderdata.h:929-941: the phasor is computed in double, stored as
//      complex<float>);
//   2. model subtraction;
//   3. weights of unselected samples are 0, then squared or set to 1 for
//      non-zero weights by the visibility weighting mode;
//   4. the imaging weight GetWeight(u / lambda, v / lambda), as float;
//   5. each correlation is multiplied by weight x imaging weight, and the
//      sums are accumulated (pol 0 for the weight sum, maximum and count);
//   6. the correlations are collapsed to one value (sum of two, or Stokes /
//      correlation `polarization` of four).
// The streamed inputs are read with evict-first loads so that L2 keeps the
// imaging-weight table; VEC selects 8- / 16-byte accesses (aligned buffers).
struct PrepAcc {
  FloatSum vws, total, corr;
  float vmax = 0.0f;
  uint32_t count = 0;
  double mat[16] = {};  // matrix correction sum (WeightSumsDev::matrix layout)
};

// AverageCorrection::Add in matrix form (averagecorrection.h:36-50) for one
// sample: 0.5 w (a^H a + b^H b) with a = G1 (x) G2, b = G2 (x) G1.  By the
// mixed-product rule a^H a = P (x) Q and b^H b = Q (x) P with the 2 x 2
// Hermitian P = G1^H G1, Q = G2^H G2, so the sum is 0.5 w (P (x) Q + Q (x) P);
// its 16 independent reals are added to mat (WeightSumsDev::matrix layout).
__device__ __forceinline__ void add_correction_matrix(const float2 *g1, const float2 *g2,
                                                      float w, double *mat) {
  // H = G^H G for G = [[g0, g1], [g2, g3]]: diagonal h0, h1 and h01
  auto herm = [](const float2 *g, float *d0, float *d1, float2 *o) {
    *d0 = g[0].x * g[0].x + g[0].y * g[0].y + g[2].x * g[2].x + g[2].y * g[2].y;
    *d1 = g[1].x * g[1].x + g[1].y * g[1].y + g[3].x * g[3].x + g[3].y * g[3].y;
    const float2 a = cm(cj(g[0]), g[1]), b = cm(cj(g[2]), g[3]);
    *o = make_float2(a.x + b.x, a.y + b.y);
  };
  float p0, p1, q0, q1;
  float2 p01, q01;
  herm(g1, &p0, &p1, &p01);
  herm(g2, &q0, &q1, &q01);
  // element (2i + k, 2j + l) of P (x) Q + Q (x) P is P_ij Q_kl + Q_ij P_kl
  auto el = [](float d0, float d1, float2 o, int i, int j) -> float2 {
    if (i == j) return make_float2(i == 0 ? d0 : d1, 0.0f);
    return i < j ? o : cj(o);
  };
  const double hw = 0.5 * (double)w;
  constexpr int kRow[10] = {0, 1, 2, 3, 0, 0, 0, 1, 1, 2};
  constexpr int kCol[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};
#pragma unroll
  for (int e = 0; e < 10; ++e) {
    const int r = kRow[e], c = kCol[e];
    const int i = r >> 1, k = r & 1, j = c >> 1, l = c & 1;
    const float2 a = cm(el(p0, p1, p01, i, j), el(q0, q1, q01, k, l));
    const float2 b = cm(el(q0, q1, q01, i, j), el(p0, p1, p01, k, l));
    if (e < 4) {
      mat[e] += hw * (double)(a.x + b.x);
    } else {
      mat[4 + 2 * (e - 4)] += hw * (double)(a.x + b.x);
      mat[5 + 2 * (e - 4)] += hw * (double)(a.y + b.y);
    }
  }
}

template <int NPOL, bool VEC>
__device__ __forceinline__ void load_weights(const float *p, float *w) {
  if constexpr (VEC && NPOL == 4) {
    const float4 t = __ldcs(reinterpret_cast<const float4 *>(p));
    w[0] = t.x; w[1] = t.y; w[2] = t.z; w[3] = t.w;
  } else if constexpr (VEC && NPOL == 2) {
    const float2 t = __ldcs(reinterpret_cast<const float2 *>(p));
    w[0] = t.x; w[1] = t.y;
  } else {
#pragma unroll
    for (int k = 0; k < NPOL; ++k) w[k] = __ldcs(p + k);
  }
}

template <int NPOL, bool VEC>
__device__ __forceinline__ void load_vis(const float2 *p, float2 *v) {
  if constexpr (VEC && NPOL >= 2) {
#pragma unroll
    for (int k = 0; k < NPOL / 2; ++k) {
      const float4 t = __ldcs(reinterpret_cast<const float4 *>(p) + k);
      v[2 * k] = make_float2(t.x, t.y);
      v[2 * k + 1] = make_float2(t.z, t.w);
    }
  } else {
#pragma unroll
    for (int k = 0; k < NPOL; ++k) v[k] = __ldcs(p + k);
  }
}

// With CORR the conjugated gains of the row's antennas are applied between
// the weighting and ApplyWeights (ApplyWeightsAndCorrections,
// msgridderdata.h:888-927, through VisibilityModifier::
// ApplyConjugatedParmResponse, visibilitymodifier.h:538-594), and for TRACE
// the correction sum |g|^2 w iw of AverageCorrection::Add
// (averagecorrection.h:36-50, g = (g2[0] conj(g1[0]) + g2[3] conj(g1[3])) / 2)
// is accumulated.  A row whose antenna or time index is outside the solution
// table sets the error flag and contributes nothing.
template <int NPOL, bool VEC, bool CORR>
__device__ __forceinline__ void prep_sample(const RowWeighting &rw, const GainTable &gt,
                                            uint32_t e, uint32_t r, uint32_t ch, uint32_t n_chan,
                                            float iw, double lambda, const double *uvw,
                                            const float2 *vis, const float *weights,
                                            const float2 *model, const uint8_t *selected,
                                            float2 *vis_out, float *weights_out,
                                            float *imaging_out, PrepAcc &acc) {
  float2 g1[4], g2[4];
  if constexpr (CORR) {
    const uint64_t a1 = gt.ant[2 * (size_t)r], a2 = gt.ant[2 * (size_t)r + 1];
    const uint64_t t = gt.tof[r];
    if (a1 >= (uint64_t)gt.n_ant || a2 >= (uint64_t)gt.n_ant || t >= (uint64_t)gt.n_times) {
      atomicOr(gt.err, 1);
      __stcs(vis_out + e, make_float2(0.0f, 0.0f));
      if (weights_out)
        for (int p = 0; p < NPOL; ++p) __stcs(weights_out + (size_t)e * NPOL + p, 0.0f);
      if (imaging_out) __stcs(imaging_out + e, iw);
      return;
    }
    const size_t off = (((size_t)t * n_chan + ch) * (size_t)gt.n_ant) * (size_t)gt.nparms;
    if (gt.nparms == 2) {
      g1[0] = gt.sol[off + a1 * 2]; g1[1] = g1[2] = make_float2(0.f, 0.f);
      g1[3] = gt.sol[off + a1 * 2 + 1];
      g2[0] = gt.sol[off + a2 * 2]; g2[1] = g2[2] = make_float2(0.f, 0.f);
      g2[3] = gt.sol[off + a2 * 2 + 1];
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        g1[k] = gt.sol[off + a1 * 4 + k];
        g2[k] = gt.sol[off + a2 * 4 + k];
      }
    }
  }
  float w[NPOL];
  float2 v[NPOL];
  load_weights<NPOL, VEC>(weights + (size_t)e * NPOL, w);
  if (rw.psf_mode == WGPU_PSF_NONE) {
    load_vis<NPOL, VEC>(vis + (size_t)e * NPOL, v);
  } else {
    float2 ph = make_float2(1.0f, 0.0f);
    if (rw.dl != 0.0 || rw.dm != 0.0) {
      const double um = uvw[3 * (size_t)r], vm = uvw[3 * (size_t)r + 1];
      const double wm = uvw[3 * (size_t)r + 2];
      const double dn =
          sqrt(__dsub_rn(__dsub_rn(1.0, __dmul_rn(rw.dl, rw.dl)), __dmul_rn(rw.dm, rw.dm))) -
          1.0;
      const double shift = __dmul_rn(
          2.0 * M_PI,
          __dadd_rn(__dadd_rn(__dmul_rn(um, rw.dl), __dmul_rn(vm, rw.dm)), __dmul_rn(wm, dn)));
      double sn, cn;
      sincos(shift / lambda, &sn, &cn);
      ph = make_float2((float)cn, (float)sn);
    }
#pragma unroll
    for (int p = 0; p < NPOL; ++p) v[p] = ph;
  }
  if (rw.subtract_model) {
    float2 m[NPOL];
    load_vis<NPOL, VEC>(model + (size_t)e * NPOL, m);
#pragma unroll
    for (int p = 0; p < NPOL; ++p) v[p] = make_float2(v[p].x - m[p].x, v[p].y - m[p].y);
  }
  const bool sel = selected == nullptr || selected[e] != 0;
#pragma unroll
  for (int p = 0; p < NPOL; ++p) {
    float wp = sel ? w[p] : 0.0f;
    if (rw.visibility_weighting == WGPU_VISW_SQUARED)
      wp = __fmul_rn(wp, wp);
    else if (rw.visibility_weighting == WGPU_VISW_UNIT && wp != 0.0f)
      wp = 1.0f;
    w[p] = wp;
  }
  if constexpr (CORR) {
    apply_conjugated_gain<NPOL>(gt.mode, v, g1, g2);
    if (gt.mode == WGPU_GAIN_TRACE) {
      const float2 a = cm(g2[0], cj(g1[0])), b = cm(g2[3], cj(g1[3]));
      const float2 g = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y + b.y));
      acc.corr.add(__fmul_rn(g.x * g.x + g.y * g.y, __fmul_rn(w[0], iw)));
    } else if (gt.sum_matrix) {
      add_correction_matrix(g1, g2, __fmul_rn(w[0], iw), acc.mat);
    }
  }
  float2 c[NPOL];
#pragma unroll
  for (int p = 0; p < NPOL; ++p) {
    const float wp = w[p];
    const float cum = __fmul_rn(wp, iw);
    const bool has = cum != 0.0f;
    if (p == 0) {
      if (has) acc.vws.add(wp);
      acc.vmax = fmaxf(acc.vmax, cum);
      acc.count += has ? 1u : 0u;
    }
    acc.total.add(cum);
    w[p] = cum;
    // rounded products: the collapse's sums must not fuse with them
    c[p] = make_float2(__fmul_rn(v[p].x, cum), __fmul_rn(v[p].y, cum));
  }
  if (weights_out) {
    float *o = weights_out + (size_t)e * NPOL;
    if constexpr (VEC && NPOL == 4)
      __stcs(reinterpret_cast<float4 *>(o), make_float4(w[0], w[1], w[2], w[3]));
    else
#pragma unroll
      for (int p = 0; p < NPOL; ++p) __stcs(o + p, w[p]);
  }
  float2 out;
  if constexpr (NPOL == 1)
    out = c[0];
  else if constexpr (NPOL == 2)
    out = ca(c[0], c[1]);
  else
    out = collapse4(c, rw.polarization);
  __stcs(vis_out + e, out);
  if (imaging_out) __stcs(imaging_out + e, iw);
}

// Block reduction of the accumulators and one set of atomics per block; with
// MAT the matrix correction sum too (warp reductions, one atomic per warp and
// value).
template <bool MAT>
__device__ void finish_prep_sums(PrepAcc &acc, WeightSumsDev *sums) {
  if constexpr (MAT) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      double v = acc.mat[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(&sums->matrix[k], v);
    }
  }
  const double s_vws = block_sum(acc.vws.value());
  const double s_total = block_sum(acc.total.value());
  const double s_count = block_sum((double)acc.count);
  const double s_corr = block_sum(acc.corr.value());
  __shared__ float wmax[kThreads / 32];
  float m = acc.vmax;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float bm = 0.0f;
    for (int k = 0; k < kThreads / 32; ++k) bm = fmaxf(bm, wmax[k]);
    if (s_vws != 0.0) atomicAdd(&sums->visibility_weight_sum, s_vws);
    if (s_total != 0.0) atomicAdd(&sums->total_weight, s_total);
    if (s_count != 0.0) atomicAdd(&sums->count, (unsigned long long)s_count);
    if (s_corr != 0.0) atomicAdd(&sums->correction, s_corr);
    // positive doubles order like their bit patterns
    if (bm > 0.0f)
      atomicMax(&sums->max_bits, (unsigned long long)__double_as_longlong((double)bm));
  }
}

// First pass over a fixed grid of blocks: samples whose imaging-weight cell is
// decided in FP32 are prepared; the others go to the pending list.
template <int NPOL, bool VEC, bool CORR>
__global__ void __launch_bounds__(kThreads, CORR ? 2 : 5) prepare_rows_fast_kernel(
    WeightGridView g, RowWeighting rw, GainTable gt, uint32_t n, uint32_t n_chan,
    const double *uvw, const ChanScale *cs, const float2 *vis, const float *weights,
    const float2 *model, const uint8_t *selected, float2 *vis_out, float *weights_out,
    float *imaging_out, WeightSumsDev *sums, Pending pend) {
  __shared__ uint32_t s_count;
  if (threadIdx.x == 0) s_count = 0;
  __syncthreads();
  PrepAcc acc;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t e = base + threadIdx.x;
    bool undecided = false;
    if (e < n) {
      const uint32_t r = e / n_chan, ch = e - r * n_chan;
      const ChanScale c = cs[ch];
      const int64_t cell = fast_cell(uvw[3 * (size_t)r], uvw[3 * (size_t)r + 1], c, g.width,
                                     g.height);
      undecided = cell == -2;
      if (!undecided)
        prep_sample<NPOL, VEC, CORR>(rw, gt, e, r, ch, n_chan, cell >= 0 ? g.gridf[cell] : 0.0f,
                                     c.lambda, uvw, vis, weights, model, selected, vis_out,
                                     weights_out, imaging_out, acc);
    }
    pending_push(pend, &s_count, undecided, e);
  }
  finish_prep_sums<CORR>(acc, sums);
  if (threadIdx.x == 0) pend.counts[blockIdx.x] = s_count;
}

// Second pass over the pending samples, with the cell of GetWeight(u, v)
// computed in double as on the host.
template <int NPOL, bool VEC, bool CORR>
__global__ void __launch_bounds__(kThreads) prepare_rows_exact_kernel(
    WeightGridView g, RowWeighting rw, GainTable gt, uint32_t n_chan, const double *uvw,
    const ChanScale *cs, const float2 *vis, const float *weights, const float2 *model,
    const uint8_t *selected, float2 *vis_out, float *weights_out, float *imaging_out,
    WeightSumsDev *sums, Pending pend) {
  const uint32_t count = pend.counts[blockIdx.x];
  const uint32_t *list = pend.idx + (size_t)blockIdx.x * pend.cap;
  PrepAcc acc;
  for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
    const uint32_t e = list[i];
    const uint32_t r = e / n_chan, ch = e - r * n_chan;
    const double lambda = cs[ch].lambda;
    const int64_t cell = uv_cell(uvw[3 * (size_t)r] / lambda, uvw[3 * (size_t)r + 1] / lambda,
                                 g.width, g.height, g.psx, g.psy);
    prep_sample<NPOL, VEC, CORR>(rw, gt, e, r, ch, n_chan, cell >= 0 ? g.gridf[cell] : 0.0f,
                                 lambda, uvw, vis, weights, model, selected, vis_out, weights_out,
                                 imaging_out, acc);
  }
  finish_prep_sums<CORR>(acc, sums);
}

__global__ void grid_to_float_kernel(const double *grid, int64_t n, float *gridf) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) gridf[i] = (float)grid[i];
}

// Launch geometry of the two-pass kernels for n samples.
struct PassShape {
  unsigned blocks;
  uint32_t cap;
};

constexpr int kMaxBlocksPerSm = 8;

// All blocks resident at once (a grid-stride loop over the samples).
PassShape pass_shape(uint32_t n, int blocks_per_sm) {
  PassShape s;
  s.blocks = (unsigned)(std::max(1, std::min(blocks_per_sm, kMaxBlocksPerSm)) * sm_count());
  const uint64_t stride = (uint64_t)s.blocks * kThreads;
  s.cap = (uint32_t)(((uint64_t)n + stride - 1) / stride * kThreads);
  return s;
}

template <typename Kernel>
int resident_blocks(Kernel k) {
  int nb = 0;
  WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kThreads, 0));
  return nb;
}

// Samples per launch (row-aligned): indices stay 32-bit.
int64_t rows_per_launch(int64_t n_chan) { return std::max<int64_t>(1, (1ll << 30) / n_chan); }

}  // namespace


WeightGridView imageweights_view(const wgpu_imageweights_t *iw_c) {
  auto *iw = const_cast<wgpu_imageweights_t *>(iw_c);
  if (iw->gridf_dirty) {
    // the float copy the row preparation samples: (float)grid, the value
    // GetWeight's result takes in the reference's float weight buffer
    const int64_t n = iw->width * (iw->height / 2);
    grid_to_float_kernel<<<blocks_for(n), kThreads, 0, iw->stream>>>(iw->grid, n, iw->gridf);
    check_launch("grid_to_float_kernel");
    WGPU_CUDA(cudaStreamSynchronize(iw->stream));
    iw->gridf_dirty = false;
  }
  WeightGridView v;
  v.grid = iw->grid;
  v.gridf = iw->gridf;
  v.width = iw->width;
  v.height = iw->height;
  v.psx = iw->psx;
  v.psy = iw->psy;
  return v;
}

RowWeighting row_weighting(const wgpu_row_weighting_t &rw) {
  RowWeighting r;
  r.psf_mode = rw.psf_mode;
  r.subtract_model = rw.subtract_model != 0;
  r.visibility_weighting = rw.visibility_weighting;
  r.polarization = rw.polarization;
  r.dl = rw.psf_dl;
  r.dm = rw.psf_dm;
  return r;
}

void add_weight_sums(const WeightSumsDev &d, wgpu_weight_sums_t *sums) {
  if (!sums) return;
  sums->visibility_weight_sum += d.visibility_weight_sum;
  sums->total_weight += d.total_weight;
  sums->gridded_visibility_count += d.count;
  double m;
  std::memcpy(&m, &d.max_bits, sizeof(m));
  if (m > sums->max_gridded_weight) sums->max_gridded_weight = m;
}

namespace {

size_t align16(size_t b) { return (b + 15) / 16 * 16; }

// Work buffer of the two-pass kernels: the channel table, the per-block
// pending counts and the pending slices of the largest launch.
struct PassWork {
  ChanScale *cs;
  uint32_t *counts;
  uint32_t *idx;
};

PassWork carve_work(void *work, int64_t n_chan) {
  char *p = (char *)work;
  PassWork w;
  w.cs = (ChanScale *)p;
  p += align16(sizeof(ChanScale) * (size_t)n_chan);
  w.counts = (uint32_t *)p;
  p += align16(sizeof(uint32_t) * (size_t)(kMaxBlocksPerSm * sm_count()));
  w.idx = (uint32_t *)p;
  return w;
}

template <typename T>
T *at(T *p, size_t k) {
  return p ? p + k : nullptr;
}

bool aligned16(const void *p) { return p == nullptr || ((uintptr_t)p & 15) == 0; }

}  // namespace

size_t pass_work_bytes(int64_t n_rows, int64_t n_chan) {
  // blocks * cap <= n + blocks * kThreads for any number of blocks
  const int64_t rows = std::min(n_rows, rows_per_launch(n_chan));
  const size_t max_blocks = (size_t)kMaxBlocksPerSm * (size_t)sm_count();
  return align16(sizeof(ChanScale) * (size_t)n_chan) + align16(sizeof(uint32_t) * max_blocks) +
         sizeof(uint32_t) * ((size_t)(rows * n_chan) + max_blocks * kThreads);
}

void launch_weight_grid(const WeightGridView &g, double *grid, double *total, int as_taper,
                        int64_t n_rows, int64_t n_chan, int n_pol, const double *uvw,
                        const double *freq, const float *weights, void *work, cudaStream_t s) {
  if (n_rows == 0 || n_chan == 0) return;
  const PassWork w = carve_work(work, n_chan);
  chan_scale_kernel<<<blocks_for(n_chan), kThreads, 0, s>>>(freq, n_chan, g.width, g.height,
                                                            g.psx, g.psy, w.cs);
  check_launch("chan_scale_kernel");
  const int64_t rpl = rows_per_launch(n_chan);
  for (int64_t r0 = 0; r0 < n_rows; r0 += rpl) {
    const int64_t rows = std::min(rpl, n_rows - r0);
    const uint32_t n = (uint32_t)(rows * n_chan);
    const size_t off = (size_t)r0 * (size_t)n_chan;
    const PassShape ps = pass_shape(n, resident_blocks(weight_grid_fast_kernel));
    const Pending pend{w.idx, w.counts, ps.cap};
    weight_grid_fast_kernel<<<ps.blocks, kThreads, 0, s>>>(
        grid, total, g.width, g.height, as_taper, n, (uint32_t)n_chan, n_pol, uvw + 3 * r0, w.cs,
        weights + off * n_pol, pend);
    check_launch("weight_grid_fast_kernel");
    weight_grid_exact_kernel<<<ps.blocks, kThreads, 0, s>>>(
        grid, total, g.width, g.height, g.psx, g.psy, as_taper, (uint32_t)n_chan, n_pol,
        uvw + 3 * r0, w.cs, weights + off * n_pol, pend);
    check_launch("weight_grid_exact_kernel");
  }
}

void launch_prepare_rows(const WeightGridView &g, const RowWeighting &rw, int n_pol,
                         int64_t n_rows, int64_t n_chan, const double *uvw, const double *freq,
                         const float2 *vis, const float *weights, const float2 *model,
                         const uint8_t *selected, float2 *vis_out, float *weights_out,
                         float *imaging_out, WeightSumsDev *sums, void *work, cudaStream_t s,
                         const GainTable *gains) {
  if (n_rows == 0 || n_chan == 0) return;
  const PassWork w = carve_work(work, n_chan);
  const GainTable gt0 = gains ? *gains : GainTable();
  chan_scale_kernel<<<blocks_for(n_chan), kThreads, 0, s>>>(freq, n_chan, g.width, g.height,
                                                            g.psx, g.psy, w.cs);
  check_launch("chan_scale_kernel");
  const bool vec = n_pol >= 2 && aligned16(vis) && aligned16(weights) && aligned16(model) &&
                   aligned16(weights_out);
  const int64_t rpl = rows_per_launch(n_chan);
  for (int64_t r0 = 0; r0 < n_rows; r0 += rpl) {
    const int64_t rows = std::min(rpl, n_rows - r0);
    const uint32_t n = (uint32_t)(rows * n_chan);
    const size_t off = (size_t)r0 * (size_t)n_chan, offp = off * (size_t)n_pol;
    const int bps = n_pol == 1 ? resident_blocks(prepare_rows_fast_kernel<1, false, false>)
                    : n_pol == 2 ? resident_blocks(prepare_rows_fast_kernel<2, true, false>)
                                 : resident_blocks(prepare_rows_fast_kernel<4, true, false>);
    // the gain table's rows start at this launch's first row
    GainTable gt = gt0;
    if (gains) {
      gt.ant = gt0.ant + 2 * r0;
      gt.tof = gt0.tof + r0;
    }
    const PassShape ps = pass_shape(n, bps);
    const Pending pend{w.idx, w.counts, ps.cap};
    const double *u = uvw + 3 * r0;
    const float2 *v = at(vis, offp), *m = at(model, offp);
    const float *wt = weights + offp;
    const uint8_t *sl = at(selected, off);
    float2 *vo = vis_out + off;
    float *wo = at(weights_out, offp), *io = at(imaging_out, off);
#define WGPU_PREP_LAUNCH(NP, VEC, CORR)                                                        \
  do {                                                                                         \
    prepare_rows_fast_kernel<NP, VEC, CORR><<<ps.blocks, kThreads, 0, s>>>(                   \
        g, rw, gt, n, (uint32_t)n_chan, u, w.cs, v, wt, m, sl, vo, wo, io, sums, pend);        \
    check_launch("prepare_rows_fast_kernel");                                                  \
    prepare_rows_exact_kernel<NP, VEC, CORR><<<ps.blocks, kThreads, 0, s>>>(                  \
        g, rw, gt, (uint32_t)n_chan, u, w.cs, v, wt, m, sl, vo, wo, io, sums, pend);           \
    check_launch("prepare_rows_exact_kernel");                                                 \
  } while (0)
#define WGPU_PREP_DISPATCH(CORR)          \
  do {                                    \
    if (n_pol == 1)                       \
      WGPU_PREP_LAUNCH(1, false, CORR);   \
    else if (n_pol == 2 && vec)           \
      WGPU_PREP_LAUNCH(2, true, CORR);    \
    else if (n_pol == 2)                  \
      WGPU_PREP_LAUNCH(2, false, CORR);   \
    else if (vec)                         \
      WGPU_PREP_LAUNCH(4, true, CORR);    \
    else                                  \
      WGPU_PREP_LAUNCH(4, false, CORR);   \
  } while (0)
    if (gains)
      WGPU_PREP_DISPATCH(true);
    else
      WGPU_PREP_DISPATCH(false);
#undef WGPU_PREP_DISPATCH
#undef WGPU_PREP_LAUNCH
  }
}

}  // namespace wgpu

// ---- C ABI ------------------------------------------------------------------

namespace {

using wgpu::Error;

template <typename F>
int weights_guarded(F &&fn) {
  try {
    wgpu::clear_failure();
    fn();
    return WGPU_OK;
  } catch (const Error &e) {
    return wgpu::report_failure(e.status, e.what());
  } catch (const std::bad_alloc &) {
    return wgpu::report_failure(WGPU_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception &e) {
    return wgpu::report_failure(WGPU_ERR_INVALID, e.what());
  }
}

// Makes the image weights' device current for the scope of a call.
struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(int dev) {
    WGPU_CUDA(cudaGetDevice(&prev));
    if (prev != dev) WGPU_CUDA(cudaSetDevice(dev));
  }
  ~DeviceScope() {
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != prev && prev >= 0) cudaSetDevice(prev);
  }
};

void *scratch(wgpu_imageweights_t *iw, int slot, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (iw->scratch_bytes[slot] < bytes) {
    WGPU_CUDA(cudaStreamSynchronize(iw->stream));
    if (iw->scratch[slot]) WGPU_CUDA(cudaFree(iw->scratch[slot]));
    iw->scratch[slot] = nullptr;
    iw->scratch_bytes[slot] = 0;
    WGPU_CUDA(cudaMalloc(&iw->scratch[slot], bytes));
    iw->scratch_bytes[slot] = bytes;
  }
  return iw->scratch[slot];
}

template <typename T>
T *upload(wgpu_imageweights_t *iw, int slot, const T *h, size_t n) {
  T *d = (T *)scratch(iw, slot, sizeof(T) * n);
  WGPU_CUDA(cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, iw->stream));
  return d;
}

int64_t grid_cells(const wgpu_imageweights_t *iw) { return iw->width * (iw->height / 2); }

bool valid_weighting(const wgpu_row_weighting_t *rw) {
  return rw && rw->psf_mode >= WGPU_PSF_NONE && rw->psf_mode <= WGPU_PSF_DIRECTION_DEPENDENT &&
         rw->visibility_weighting >= WGPU_VISW_NORMAL &&
         rw->visibility_weighting <= WGPU_VISW_UNIT && rw->polarization >= 0 &&
         rw->polarization <= 7;
}

void grid_device(wgpu_imageweights_t *iw, size_t n_rows, size_t n_chan, size_t n_pol,
                 const double *du, const double *df, const float *dw) {
  void *work = scratch(iw, 9, wgpu::pass_work_bytes((int64_t)n_rows, (int64_t)n_chan));
  iw->gridf_dirty = true;
  wgpu::WeightGridView g;
  g.grid = iw->grid;
  g.gridf = nullptr;
  g.width = iw->width;
  g.height = iw->height;
  g.psx = iw->psx;
  g.psy = iw->psy;
  wgpu::launch_weight_grid(g, iw->grid, iw->sums, iw->as_taper ? 1 : 0, (int64_t)n_rows,
                           (int64_t)n_chan, (int)n_pol, du, df, dw, work, iw->stream);
  WGPU_CUDA(cudaStreamSynchronize(iw->stream));
}

// The row preparation on device buffers; sums (device, zeroed here) are read
// back and added to the caller's.
void prepare_device(wgpu_imageweights_t *iw, const wgpu_row_weighting_t *rw, size_t n_pol,
                    size_t n_rows, size_t n_chan, const double *du, const double *df,
                    const float2 *dv, const float *dw, const float2 *dm, const uint8_t *ds,
                    float2 *dvo, float *dwo, float *dio, wgpu_weight_sums_t *sums) {
  auto *dsum = (wgpu::WeightSumsDev *)scratch(iw, 7, sizeof(wgpu::WeightSumsDev));
  void *work = scratch(iw, 8, wgpu::pass_work_bytes((int64_t)n_rows, (int64_t)n_chan));
  const wgpu::WeightGridView view = wgpu::imageweights_view(iw);
  WGPU_CUDA(cudaMemsetAsync(dsum, 0, sizeof(wgpu::WeightSumsDev), iw->stream));
  wgpu::launch_prepare_rows(view, wgpu::row_weighting(*rw), (int)n_pol, (int64_t)n_rows,
                            (int64_t)n_chan, du, df, dv, dw, dm, ds, dvo, dwo, dio, dsum, work,
                            iw->stream);
  wgpu::WeightSumsDev hs;
  WGPU_CUDA(cudaMemcpyAsync(&hs, dsum, sizeof(hs), cudaMemcpyDeviceToHost, iw->stream));
  WGPU_CUDA(cudaStreamSynchronize(iw->stream));
  wgpu::add_weight_sums(hs, sums);
}

int check_prepare_args(const wgpu_imageweights_t *iw, const wgpu_row_weighting_t *rw,
                       size_t n_pol, size_t n_rows, size_t n_chan, const void *uvw,
                       const void *freq, const void *vis, const void *weights,
                       const void *model, const void *vis_out) {
  if (!iw) return wgpu::report_failure(WGPU_ERR_INVALID, "null image weights");
  if (!valid_weighting(rw)) return wgpu::report_failure(WGPU_ERR_INVALID, "invalid row weighting");
  if (n_pol != 1 && n_pol != 2 && n_pol != 4)
    return wgpu::report_failure(WGPU_ERR_INVALID, "n_pol must be 1, 2 or 4");
  if (n_rows && n_chan &&
      (!uvw || !freq || !weights || !vis_out || (rw->psf_mode == WGPU_PSF_NONE && !vis) ||
       (rw->subtract_model && !model)))
    return wgpu::report_failure(WGPU_ERR_INVALID, "null data pointer");
  return WGPU_OK;
}

}  // namespace

extern "C" {

int wgpu_imageweights_create(int mode, double briggs_robustness, size_t image_width,
                             size_t image_height, double pixel_scale_x, double pixel_scale_y,
                             int weights_as_taper, double super_weight,
                             wgpu_imageweights_t **out) {
  if (!out) return wgpu::report_failure(WGPU_ERR_INVALID, "null output");
  *out = nullptr;
  if (mode < WGPU_WEIGHT_NATURAL || mode > WGPU_WEIGHT_BRIGGS)
    return wgpu::report_failure(WGPU_ERR_INVALID, "invalid weighting mode");
  if (!(pixel_scale_x > 0) || !(pixel_scale_y > 0) || !(super_weight > 0))
    return wgpu::report_failure(WGPU_ERR_INVALID, "pixel scales and super weight must be > 0");
  // imageweights.cpp:34-49: round(size / superWeight), made even
  int64_t w = (int64_t)std::round((double)image_width / super_weight);
  int64_t h = (int64_t)std::round((double)image_height / super_weight);
  if (w % 2 != 0) ++w;
  if (h % 2 != 0) ++h;
  if (w < 2 || h < 2 || w > (1 << 20) || h > (1 << 20))
    return wgpu::report_failure(WGPU_ERR_INVALID, "weight grid size out of range");
  int n_dev = 0;
  if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev == 0) {
    cudaGetLastError();
    return wgpu::report_failure(WGPU_ERR_CUDA, "no CUDA device");
  }
  auto *iw = new wgpu_imageweights();
  iw->mode = mode;
  iw->robustness = briggs_robustness;
  iw->width = w;
  iw->height = h;
  iw->psx = pixel_scale_x;
  iw->psy = pixel_scale_y;
  iw->as_taper = weights_as_taper != 0;
  const int st = weights_guarded([&] {
    WGPU_CUDA(cudaGetDevice(&iw->device));
    WGPU_CUDA(cudaStreamCreateWithFlags(&iw->stream, cudaStreamNonBlocking));
    WGPU_CUDA(cudaMalloc(&iw->grid, sizeof(double) * (size_t)grid_cells(iw)));
    WGPU_CUDA(cudaMalloc(&iw->gridf, sizeof(float) * (size_t)grid_cells(iw)));
    WGPU_CUDA(cudaMalloc(&iw->sums, sizeof(double) * 2));
    WGPU_CUDA(cudaMalloc(&iw->partials, sizeof(double) * wgpu::kReduceBlocks));
    WGPU_CUDA(cudaMemsetAsync(iw->grid, 0, sizeof(double) * (size_t)grid_cells(iw), iw->stream));
    WGPU_CUDA(cudaMemsetAsync(iw->sums, 0, sizeof(double) * 2, iw->stream));
    WGPU_CUDA(cudaStreamSynchronize(iw->stream));
  });
  if (st != WGPU_OK) {
    wgpu_imageweights_destroy(iw);
    return st;
  }
  *out = iw;
  return WGPU_OK;
}

void wgpu_imageweights_destroy(wgpu_imageweights_t *iw) {
  if (!iw) return;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != iw->device) cudaSetDevice(iw->device);
  if (iw->stream) cudaStreamSynchronize(iw->stream);
  for (int k = 0; k < wgpu_imageweights::kScratch; ++k)
    if (iw->scratch[k]) cudaFree(iw->scratch[k]);
  if (iw->grid) cudaFree(iw->grid);
  if (iw->gridf) cudaFree(iw->gridf);
  if (iw->sums) cudaFree(iw->sums);
  if (iw->partials) cudaFree(iw->partials);
  if (iw->stream) cudaStreamDestroy(iw->stream);
  if (prev >= 0 && prev != iw->device) cudaSetDevice(prev);
  delete iw;
}

int wgpu_imageweights_grid(wgpu_imageweights_t *iw, size_t n_rows, size_t n_chan, size_t n_pol,
                           const double *uvw, const double *freq, const float *weights) {
  if (!iw) return wgpu::report_failure(WGPU_ERR_INVALID, "null image weights");
  if (n_pol < 1 || n_pol > 4)
    return wgpu::report_failure(WGPU_ERR_INVALID, "n_pol must be 1 to 4");
  if (n_rows && n_chan && (!uvw || !freq || !weights))
    return wgpu::report_failure(WGPU_ERR_INVALID, "null data pointer");
  return weights_guarded([&] {
    if (iw->finished) throw Error(WGPU_ERR_STATE, "Grid() after FinishGridding()");
    if (n_rows == 0 || n_chan == 0) return;
    DeviceScope scope(iw->device);
    const double *du = upload(iw, 0, uvw, 3 * n_rows);
    const double *df = upload(iw, 1, freq, n_chan);
    const float *dw = upload(iw, 2, weights, n_rows * n_chan * n_pol);
    grid_device(iw, n_rows, n_chan, n_pol, du, df, dw);
  });
}

int wgpu_imageweights_grid_device(wgpu_imageweights_t *iw, size_t n_rows, size_t n_chan,
                                  size_t n_pol, const double *d_uvw, const double *d_freq,
                                  const float *d_weights) {
  if (!iw) return wgpu::report_failure(WGPU_ERR_INVALID, "null image weights");
  if (n_pol < 1 || n_pol > 4)
    return wgpu::report_failure(WGPU_ERR_INVALID, "n_pol must be 1 to 4");
  if (n_rows && n_chan && (!d_uvw || !d_freq || !d_weights))
    return wgpu::report_failure(WGPU_ERR_INVALID, "null data pointer");
  return weights_guarded([&] {
    if (iw->finished) throw Error(WGPU_ERR_STATE, "Grid() after FinishGridding()");
    if (n_rows == 0 || n_chan == 0) return;
    DeviceScope scope(iw->device);
    grid_device(iw, n_rows, n_chan, n_pol, d_uvw, d_freq, d_weights);
  });
}

void *wgpu_imageweights_stream(wgpu_imageweights_t *iw) { return iw ? iw->stream : nullptr; }

int wgpu_imageweights_finish(wgpu_imageweights_t *iw) {
  if (!iw) return wgpu::report_failure(WGPU_ERR_INVALID, "null image weights");
  return weights_guarded([&] {
    if (iw->finished) throw Error(WGPU_ERR_STATE, "FinishGridding() called twice");
    DeviceScope scope(iw->device);
    const int64_t n = grid_cells(iw);
    double s_sq = 0.0;
    if (iw->mode == WGPU_WEIGHT_BRIGGS) {
      // imageweights.cpp:120-128: avgW = sum(val^2) / totalSum,
      // sSq = (5 * 10^-robustness)^2 / avgW
      wgpu::sum_sq_partials_kernel<<<wgpu::kReduceBlocks, wgpu::kThreads, 0, iw->stream>>>(
          iw->grid, n, iw->partials);
      wgpu::check_launch("sum_sq_partials_kernel");
      wgpu::sum_partials_kernel<<<1, wgpu::kThreads, 0, iw->stream>>>(
          iw->partials, wgpu::kReduceBlocks, iw->sums + 1);
      wgpu::check_launch("sum_partials_kernel");
      double h[2];
      WGPU_CUDA(cudaMemcpyAsync(h, iw->sums, sizeof(h), cudaMemcpyDeviceToHost, iw->stream));
      WGPU_CUDA(cudaStreamSynchronize(iw->stream));
      const double avg_w = h[1] / h[0];
      const double numerator_sqrt = 5.0 * std::exp((-M_LN10) * iw->robustness);
      s_sq = numerator_sqrt * numerator_sqrt / avg_w;
    }
    wgpu::weight_finish_kernel<<<wgpu::blocks_for(n), wgpu::kThreads, 0, iw->stream>>>(
        iw->grid, n, iw->mode, s_sq);
    wgpu::check_launch("weight_finish_kernel");
    WGPU_CUDA(cudaStreamSynchronize(iw->stream));
    iw->finished = true;
    iw->gridf_dirty = true;
  });
}

int wgpu_imageweights_taper(wgpu_imageweights_t *iw, int kind, double a, double b) {
  if (!iw) return wgpu::report_failure(WGPU_ERR_INVALID, "null image weights");
  if (kind < WGPU_TAPER_MIN_UV || kind > WGPU_TAPER_RANK_FILTER)
    return wgpu::report_failure(WGPU_ERR_INVALID, "invalid taper kind");
  if (kind == WGPU_TAPER_RANK_FILTER && !(b >= 0 && b <= 256 && b == std::floor(b)))
    return wgpu::report_failure(WGPU_ERR_INVALID, "rank filter window must be 0 to 256");
  if (kind == WGPU_TAPER_GAUSSIAN && !(a != 0))
    return wgpu::report_failure(WGPU_ERR_INVALID, "Gaussian taper beam size must be non-zero");
  return weights_guarded([&] {
    DeviceScope scope(iw->device);
    const int64_t n = grid_cells(iw);
    if (kind == WGPU_TAPER_RANK_FILTER) {
      double *src = (double *)scratch(iw, 3, sizeof(double) * (size_t)n);
      WGPU_CUDA(cudaMemcpyAsync(src, iw->grid, sizeof(double) * (size_t)n,
                                cudaMemcpyDeviceToDevice, iw->stream));
      wgpu::rank_filter_kernel<<<wgpu::blocks_for(n), wgpu::kThreads, 0, iw->stream>>>(
          src, iw->grid, iw->width, iw->height / 2, a, (int64_t)b);
      wgpu::check_launch("rank_filter_kernel");
      iw->gridf_dirty = true;
    } else {
      double pa = a;
      if (kind == WGPU_TAPER_GAUSSIAN) {
        // imageweights.cpp:328-338: half-power uv radius, in long double the
        // sigma-to-half-power factor, then -2 sigma^2
        const double half_power_uv = 1.0 / (a * 2.0 * M_PI);
        const long double sigma_to_hp = 2.0L * sqrtl(2.0L * logl(2.0L));
        double m = half_power_uv * sigma_to_hp;
        m *= -2.0 * m;
        pa = m;
      }
      wgpu::weight_taper_kernel<<<wgpu::blocks_for(n), wgpu::kThreads, 0, iw->stream>>>(
          iw->grid, iw->width, iw->height, iw->psx, iw->psy, kind, pa, b);
      wgpu::check_launch("weight_taper_kernel");
      iw->gridf_dirty = true;
    }
    WGPU_CUDA(cudaStreamSynchronize(iw->stream));
  });
}

int wgpu_imageweights_set_all(wgpu_imageweights_t *iw, double value) {
  if (!iw) return wgpu::report_failure(WGPU_ERR_INVALID, "null image weights");
  return weights_guarded([&] {
    DeviceScope scope(iw->device);
    const int64_t n = grid_cells(iw);
    wgpu::weight_fill_kernel<<<wgpu::blocks_for(n), wgpu::kThreads, 0, iw->stream>>>(
        iw->grid, n, value);
    wgpu::check_launch("weight_fill_kernel");
    iw->gridf_dirty = true;
    WGPU_CUDA(cudaStreamSynchronize(iw->stream));
  });
}

int wgpu_imageweights_get(const wgpu_imageweights_t *iw_c, int mirrored, double *out) {
  if (!iw_c || !out) return wgpu::report_failure(WGPU_ERR_INVALID, "null argument");
  auto *iw = const_cast<wgpu_imageweights_t *>(iw_c);
  return weights_guarded([&] {
    DeviceScope scope(iw->device);
    const int64_t n = grid_cells(iw);
    if (!mirrored) {
      WGPU_CUDA(cudaMemcpyAsync(out, iw->grid, sizeof(double) * (size_t)n,
                                cudaMemcpyDeviceToHost, iw->stream));
    } else {
      double *img = (double *)scratch(iw, 4, sizeof(double) * (size_t)(2 * n));
      wgpu::weight_mirror_kernel<<<wgpu::blocks_for(n), wgpu::kThreads, 0, iw->stream>>>(
          iw->grid, iw->width, iw->height, img);
      wgpu::check_launch("weight_mirror_kernel");
      WGPU_CUDA(cudaMemcpyAsync(out, img, sizeof(double) * (size_t)(2 * n),
                                cudaMemcpyDeviceToHost, iw->stream));
    }
    WGPU_CUDA(cudaStreamSynchronize(iw->stream));
  });
}

int wgpu_imageweights_info(const wgpu_imageweights_t *iw, size_t *width, size_t *height,
                           double *total_sum) {
  if (!iw) return wgpu::report_failure(WGPU_ERR_INVALID, "null image weights");
  return weights_guarded([&] {
    if (width) *width = (size_t)iw->width;
    if (height) *height = (size_t)iw->height;
    if (total_sum) {
      DeviceScope scope(iw->device);
      WGPU_CUDA(cudaMemcpyAsync(total_sum, iw->sums, sizeof(double), cudaMemcpyDeviceToHost,
                                iw->stream));
      WGPU_CUDA(cudaStreamSynchronize(iw->stream));
    }
  });
}

int wgpu_imageweights_sample(const wgpu_imageweights_t *iw_c, size_t n, const double *u,
                             const double *v, double *out) {
  if (!iw_c || (n && (!u || !v || !out)))
    return wgpu::report_failure(WGPU_ERR_INVALID, "null argument");
  auto *iw = const_cast<wgpu_imageweights_t *>(iw_c);
  return weights_guarded([&] {
    if (n == 0) return;
    DeviceScope scope(iw->device);
    const double *du = upload(iw, 0, u, n);
    const double *dv = upload(iw, 1, v, n);
    double *dout = (double *)scratch(iw, 2, sizeof(double) * n);
    wgpu::weight_sample_kernel<<<wgpu::blocks_for((int64_t)n), wgpu::kThreads, 0, iw->stream>>>(
        iw->grid, iw->width, iw->height, iw->psx, iw->psy, (int64_t)n, du, dv, dout);
    wgpu::check_launch("weight_sample_kernel");
    WGPU_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, iw->stream));
    WGPU_CUDA(cudaStreamSynchronize(iw->stream));
  });
}

int wgpu_prepare_rows(const wgpu_imageweights_t *iw_c, const wgpu_row_weighting_t *rw,
                      size_t n_pol, size_t n_rows, size_t n_chan, const double *uvw,
                      const double *freq, const float *vis, const float *weights,
                      const float *model, const uint8_t *selected, float *vis_out,
                      float *weights_out, float *imaging_weights_out,
                      wgpu_weight_sums_t *sums) {
  const int st = check_prepare_args(iw_c, rw, n_pol, n_rows, n_chan, uvw, freq, vis, weights,
                                    model, vis_out);
  if (st != WGPU_OK) return st;
  auto *iw = const_cast<wgpu_imageweights_t *>(iw_c);
  return weights_guarded([&] {
    if (n_rows == 0 || n_chan == 0) return;
    DeviceScope scope(iw->device);
    const size_t n = n_rows * n_chan, nc = n * n_pol;
    const double *du = upload(iw, 0, uvw, 3 * n_rows);
    const double *df = upload(iw, 1, freq, n_chan);
    const float *dw = upload(iw, 2, weights, nc);
    const float2 *dv =
        rw->psf_mode == WGPU_PSF_NONE ? (const float2 *)upload(iw, 3, vis, 2 * nc) : nullptr;
    const float2 *dm = rw->subtract_model ? (const float2 *)upload(iw, 4, model, 2 * nc) : nullptr;
    const uint8_t *ds = selected ? upload(iw, 5, selected, n) : nullptr;
    // the outputs share one buffer: vis_out, weights_out, imaging weights
    char *o = (char *)scratch(iw, 6, 8 * n + 4 * nc + 4 * n);
    float2 *dvo = (float2 *)o;
    float *dwo = (float *)(o + 8 * n);
    float *dio = (float *)(o + 8 * n + 4 * nc);
    prepare_device(iw, rw, n_pol, n_rows, n_chan, du, df, dv, dw, dm, ds, dvo,
                   weights_out ? dwo : nullptr, imaging_weights_out ? dio : nullptr, sums);
    WGPU_CUDA(cudaMemcpyAsync(vis_out, dvo, 8 * n, cudaMemcpyDeviceToHost, iw->stream));
    if (weights_out)
      WGPU_CUDA(cudaMemcpyAsync(weights_out, dwo, 4 * nc, cudaMemcpyDeviceToHost, iw->stream));
    if (imaging_weights_out)
      WGPU_CUDA(
          cudaMemcpyAsync(imaging_weights_out, dio, 4 * n, cudaMemcpyDeviceToHost, iw->stream));
    WGPU_CUDA(cudaStreamSynchronize(iw->stream));
  });
}

int wgpu_prepare_rows_device(const wgpu_imageweights_t *iw_c, const wgpu_row_weighting_t *rw,
                             size_t n_pol, size_t n_rows, size_t n_chan, const double *d_uvw,
                             const double *d_freq, const float *d_vis, const float *d_weights,
                             const float *d_model, const uint8_t *d_selected, float *d_vis_out,
                             float *d_weights_out, float *d_imaging_weights_out,
                             wgpu_weight_sums_t *sums) {
  const int st = check_prepare_args(iw_c, rw, n_pol, n_rows, n_chan, d_uvw, d_freq, d_vis,
                                    d_weights, d_model, d_vis_out);
  if (st != WGPU_OK) return st;
  auto *iw = const_cast<wgpu_imageweights_t *>(iw_c);
  return weights_guarded([&] {
    if (n_rows == 0 || n_chan == 0) return;
    DeviceScope scope(iw->device);
    prepare_device(iw, rw, n_pol, n_rows, n_chan, d_uvw, d_freq,
                   rw->psf_mode == WGPU_PSF_NONE ? (const float2 *)d_vis : nullptr, d_weights,
                   rw->subtract_model ? (const float2 *)d_model : nullptr, d_selected,
                   (float2 *)d_vis_out, d_weights_out, d_imaging_weights_out, sums);
  });
}

}  // extern "C"
