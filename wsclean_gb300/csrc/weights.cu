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
  double *sums = nullptr;      // [0] gridded weight sum, [1] sum of squares
  double *partials = nullptr;  // per-block partial sums of the reductions
  static constexpr int kScratch = 8;
  void *scratch[kScratch] = {};
  size_t scratch_bytes[kScratch] = {};
};

namespace wgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kReduceBlocks = 1024;  // fixed, so reductions add in a fixed order

unsigned blocks_for(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

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

// ImageWeights::Grid(MSProvider &, BandData) (imageweights.cpp:75-112), one
// thread per (row, channel): the row's (u, v) is reflected into v >= 0, scaled
// by the channel's wavelength, and each correlation's weight (1 for a
// non-zero weight when the weights are a taper) is added to the cell.
__global__ void weight_grid_kernel(double *grid, double *total, int64_t W, int64_t H, double psx,
                                   double psy, int as_taper, int64_t n_rows, int64_t n_chan,
                                   int n_pol, const double *uvw, const double *freq,
                                   const float *weights) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double local = 0.0;
  if (e < n_rows * n_chan) {
    const int64_t r = e / n_chan, ch = e - r * n_chan;
    double um = uvw[3 * r], vm = uvw[3 * r + 1];
    if (vm < 0.0) {
      um = -um;
      vm = -vm;
    }
    const double lambda = kSpeedOfLight / freq[ch];
    const int64_t cell = uv_cell(um / lambda, vm / lambda, W, H, psx, psy);
    if (cell >= 0) {
      for (int p = 0; p < n_pol; ++p) {
        float w = weights[e * n_pol + p];
        if (as_taper && w != 0.0f) w = 1.0f;
        if (w != 0.0f) {
          atomicAdd(grid + cell, (double)w);
          local += (double)w;
        }
      }
    }
  }
  const double t = block_sum(local);
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
// (msgridderdata.h:36-52, 760-789, 826-886), one thread per (row, channel):
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
template <int NPOL>
__global__ void prepare_rows_kernel(WeightGridView g, RowWeighting rw, int64_t n_rows,
                                    int64_t n_chan, const double *uvw, const double *freq,
                                    const float2 *vis, const float *weights,
                                    const float2 *model, const uint8_t *selected,
                                    float2 *vis_out, float *weights_out, float *imaging_out,
                                    WeightSumsDev *sums) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double vws = 0.0, total = 0.0, vmax = 0.0, count = 0.0;
  if (e < n_rows * n_chan) {
    const int64_t r = e / n_chan, ch = e - r * n_chan;
    const double um = uvw[3 * r], vm = uvw[3 * r + 1], wm = uvw[3 * r + 2];
    const double lambda = kSpeedOfLight / freq[ch];
    const int64_t cell = uv_cell(um / lambda, vm / lambda, g.width, g.height, g.psx, g.psy);
    const float iw = cell >= 0 ? (float)g.grid[cell] : 0.0f;
    float2 phasor = make_float2(1.0f, 0.0f);
    if (rw.psf_mode != WGPU_PSF_NONE && (rw.dl != 0.0 || rw.dm != 0.0)) {
      const double dn =
          sqrt(__dsub_rn(__dsub_rn(1.0, __dmul_rn(rw.dl, rw.dl)), __dmul_rn(rw.dm, rw.dm))) -
          1.0;
      const double shift = __dmul_rn(
          2.0 * M_PI,
          __dadd_rn(__dadd_rn(__dmul_rn(um, rw.dl), __dmul_rn(vm, rw.dm)), __dmul_rn(wm, dn)));
      double sn, cn;
      sincos(shift / lambda, &sn, &cn);
      phasor = make_float2((float)cn, (float)sn);
    }
    const bool sel = selected == nullptr || selected[e] != 0;
    float2 c[NPOL];
#pragma unroll
    for (int p = 0; p < NPOL; ++p) {
      const int64_t i = e * NPOL + p;
      float2 v = rw.psf_mode != WGPU_PSF_NONE ? phasor : vis[i];
      if (rw.subtract_model) {
        const float2 m = model[i];
        v = make_float2(v.x - m.x, v.y - m.y);
      }
      float w = sel ? weights[i] : 0.0f;
      if (rw.visibility_weighting == WGPU_VISW_SQUARED)
        w = w * w;
      else if (rw.visibility_weighting == WGPU_VISW_UNIT && w != 0.0f)
        w = 1.0f;
      const float cum = w * iw;
      const bool has = cum != 0.0f;
      if (p == 0) {
        vws += (double)(has ? w : 0.0f);
        vmax = fmax(vmax, (double)cum);
        count += has ? 1.0 : 0.0;
      }
      total += (double)cum;
      if (weights_out) weights_out[i] = cum;
      c[p] = make_float2(v.x * cum, v.y * cum);
    }
    float2 out;
    if (NPOL == 1)
      out = c[0];
    else if (NPOL == 2)
      out = ca(c[0], c[NPOL - 1]);
    else
      out = collapse4(c, rw.polarization);
    vis_out[e] = out;
    if (imaging_out) imaging_out[e] = iw;
  }
  const double s_vws = block_sum(vws);
  const double s_total = block_sum(total);
  const double s_count = block_sum(count);
  // block maximum of the non-negative per-thread maxima
  __shared__ double wmax[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) vmax = fmax(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = vmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int k = 0; k < kThreads / 32; ++k) m = fmax(m, wmax[k]);
    if (s_vws != 0.0) atomicAdd(&sums->visibility_weight_sum, s_vws);
    if (s_total != 0.0) atomicAdd(&sums->total_weight, s_total);
    if (s_count != 0.0) atomicAdd(&sums->count, (unsigned long long)s_count);
    // positive doubles order like their bit patterns
    if (m > 0.0) atomicMax(&sums->max_bits, (unsigned long long)__double_as_longlong(m));
  }
}

}  // namespace

WeightGridView imageweights_view(const wgpu_imageweights_t *iw) {
  WeightGridView v;
  v.grid = iw->grid;
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
  r.dn = 0.0;  // formed on the device, rounded like the host expression
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

void launch_prepare_rows(const WeightGridView &g, const RowWeighting &rw, int n_pol,
                         int64_t n_rows, int64_t n_chan, const double *uvw, const double *freq,
                         const float2 *vis, const float *weights, const float2 *model,
                         const uint8_t *selected, float2 *vis_out, float *weights_out,
                         float *imaging_out, WeightSumsDev *sums, cudaStream_t s) {
  const int64_t n = n_rows * n_chan;
  if (n == 0) return;
  const unsigned nb = blocks_for(n);
  switch (n_pol) {
    case 1:
      prepare_rows_kernel<1><<<nb, kThreads, 0, s>>>(g, rw, n_rows, n_chan, uvw, freq, vis,
                                                      weights, model, selected, vis_out,
                                                      weights_out, imaging_out, sums);
      break;
    case 2:
      prepare_rows_kernel<2><<<nb, kThreads, 0, s>>>(g, rw, n_rows, n_chan, uvw, freq, vis,
                                                      weights, model, selected, vis_out,
                                                      weights_out, imaging_out, sums);
      break;
    default:
      prepare_rows_kernel<4><<<nb, kThreads, 0, s>>>(g, rw, n_rows, n_chan, uvw, freq, vis,
                                                      weights, model, selected, vis_out,
                                                      weights_out, imaging_out, sums);
      break;
  }
  check_launch("prepare_rows_kernel");
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
  const int64_t n = (int64_t)(n_rows * n_chan);
  wgpu::weight_grid_kernel<<<wgpu::blocks_for(n), wgpu::kThreads, 0, iw->stream>>>(
      iw->grid, iw->sums, iw->width, iw->height, iw->psx, iw->psy, iw->as_taper ? 1 : 0,
      (int64_t)n_rows, (int64_t)n_chan, (int)n_pol, du, df, dw);
  wgpu::check_launch("weight_grid_kernel");
  WGPU_CUDA(cudaStreamSynchronize(iw->stream));
}

// The row preparation on device buffers; sums (device, zeroed here) are read
// back and added to the caller's.
void prepare_device(wgpu_imageweights_t *iw, const wgpu_row_weighting_t *rw, size_t n_pol,
                    size_t n_rows, size_t n_chan, const double *du, const double *df,
                    const float2 *dv, const float *dw, const float2 *dm, const uint8_t *ds,
                    float2 *dvo, float *dwo, float *dio, wgpu_weight_sums_t *sums) {
  auto *dsum = (wgpu::WeightSumsDev *)scratch(iw, 7, sizeof(wgpu::WeightSumsDev));
  WGPU_CUDA(cudaMemsetAsync(dsum, 0, sizeof(wgpu::WeightSumsDev), iw->stream));
  wgpu::launch_prepare_rows(wgpu::imageweights_view(iw), wgpu::row_weighting(*rw), (int)n_pol,
                            (int64_t)n_rows, (int64_t)n_chan, du, df, dv, dw, dm, ds, dvo, dwo,
                            dio, dsum, iw->stream);
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
