// Planner: chooses grid size, ES kernel and w-planes for one gridding call.
//
// The reference hands epsilon, sigma_min = 1.1 and sigma_max = 2.0 to ducc0
// (wgridder/gridder_simple.h:57-58, :217-225), which picks the kernel and the
// plane count internally.  Here the choice is made from the ES-kernel table
// derived by wsclean_gb300/kernel_table.py and a cost model of the GPU
// pipeline (cell updates for gridding, bytes moved per w-plane for the FFT
// passes).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "es_table.h"
#include "wgpu_internal.h"

namespace wgpu {

namespace {

bool is_smooth235(int64_t k) {
  for (int p : {2, 3, 5})
    while (k % p == 0) k /= p;
  return k == 1;
}

struct GaussLegendre {
  static constexpr int kN = 256;  // positive half of a 512-point rule
  double x[kN], w[kN];
  GaussLegendre() {
    const int n = 2 * kN;
    for (int i = 0; i < kN; ++i) {
      double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
      double dp = 1.0;
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
      x[i] = z;
      w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
  }
};

const GaussLegendre &gl() {
  static const GaussLegendre g;
  return g;
}

// Throughput constants of the cost model (cell updates/s for the stencil
// kernels, bytes/s for the FFT passes), measured on GB300 on the 8192^2
// wide-field workload: gridding + degridding 484 G cell updates in 0.76 s,
// the FFT passes of both directions 677 GB in 0.48 s.
constexpr double kCellRate = 6.3e11;
constexpr double kByteRate = 1.4e12;

// Supports above 8 use the gridding kernel without register runs (every
// read adds its whole footprint into shared memory); measured on the 8192^2
// wide-field workload its plans took 2.4 times as long as the W = 8 plan
// (1379 and 1366 ms against 582 ms per bound inversion + prediction).
constexpr double kWideSupportFactor = 2.4;

// Relative FP32 round-off of the gridded planes per unit of correction
// amplification; measured on GB300 as 2-3e-8 (random visibilities, 2D and 3D
// plans), rounded up.
constexpr double kFp32Noise = 5e-8;

}  // namespace

double es_kernel(double beta, double z) {
  if (!(std::fabs(z) < 1.0)) return 0.0;
  return std::exp(beta * (std::sqrt(1.0 - z * z) - 1.0));
}

void es_quadrature(double beta, double *z, double *g) {
  const GaussLegendre &q = gl();
  for (int i = 0; i < GaussLegendre::kN; ++i) {
    z[i] = q.x[i];
    g[i] = q.w[i] * es_kernel(beta, q.x[i]);
  }
}

double es_fourier(double beta, int support, double f) {
  const GaussLegendre &g = gl();
  double acc = 0.0;
  for (int i = 0; i < GaussLegendre::kN; ++i)
    acc += g.w[i] * es_kernel(beta, g.x[i]) *
           std::cos(M_PI * f * support * g.x[i]);
  return support * acc;
}

int64_t good_fft_size(int64_t n, int64_t multiple) {
  int64_t k = (n + multiple - 1) / multiple;
  if (k < 2) k = 2;
  while (!is_smooth235(k)) ++k;
  return k * multiple;
}

static bool try_decompose(int64_t n, int64_t *n1, int64_t *n2) {
  // n = n1 * n2 with both factors <= 256, n2 >= n1, as balanced as possible.
  int64_t best1 = -1;
  for (int64_t a = 1; a <= 256; ++a) {
    if (n % a) continue;
    const int64_t b = n / a;
    if (b > 256 || b < a) continue;
    best1 = a;  // increasing a -> more balanced
  }
  if (best1 < 0) return false;
  *n1 = best1;
  *n2 = n / best1;
  return true;
}

void fft_decompose(int64_t n, int64_t *n1, int64_t *n2) {
  if (!try_decompose(n, n1, n2))
    throw Error(WGPU_ERR_INVALID, "grid size cannot be split for the column FFT");
}

void nm1_range(int64_t width, int64_t height, double dl, double dm,
               double l_shift, double m_shift, double *lo, double *hi) {
  // Pixel (x, y) sits at l = (width/2 - x) dl + l_shift, m = (y - height/2) dm
  // + m_shift (gridding/directmsgridder.cpp:113-124 with the wrap of :70-82).
  const double l_a = (double)(width / 2 - (width - 1)) * dl + l_shift;
  const double l_b = (double)(width / 2) * dl + l_shift;
  const double m_a = (double)(-(height / 2)) * dm + m_shift;
  const double m_b = (double)(height - 1 - height / 2) * dm + m_shift;
  auto nm1 = [](double l, double m) {
    const double r2 = l * l + m * m;
    if (r2 >= 1.0) return -1.0;
    return -r2 / (std::sqrt(1.0 - r2) + 1.0);
  };
  double mn = std::min(std::min(nm1(l_a, m_a), nm1(l_a, m_b)),
                       std::min(nm1(l_b, m_a), nm1(l_b, m_b)));
  const double lc = std::min(std::max(0.0, std::min(l_a, l_b)), std::max(l_a, l_b));
  const double mc = std::min(std::max(0.0, std::min(m_a, m_b)), std::max(m_a, m_b));
  double mx = nm1(lc, mc);
  *lo = mn;
  *hi = mx;
}

namespace {

void check_request(const wgpu_plan_request_t &req) {
  if (req.width < 2 || req.height < 2 || (req.width & 1) || (req.height & 1))
    throw Error(WGPU_ERR_INVALID, "trimmed image dimensions must be even and >= 2");
  if (!(req.dl > 0.0) || !(req.dm > 0.0))
    throw Error(WGPU_ERR_INVALID, "pixel sizes must be positive");
  if (!(req.epsilon > 0.0))
    throw Error(WGPU_ERR_INVALID, "epsilon must be positive");
  if (!(req.w_max >= req.w_min))
    throw Error(WGPU_ERR_INVALID, "w_max < w_min");
}

// Every table entry within sigma_min..sigma_max (and the forced fields) whose
// error estimate meets epsilon, as a plan without its plane batch, in table
// order.  `fallback` receives the most accurate entry whose grid the row and
// column transforms take, whatever its estimate.
std::vector<wgpu_plan_t> feasible_plans(const wgpu_plan_request_t &req,
                                        const EsKernelEntry **fallback, double *fallback_err) {
  const double smin = req.sigma_min > 0 ? req.sigma_min : 1.1;
  const double smax = req.sigma_max > 0 ? req.sigma_max : 2.0;
  double lo, hi;
  nm1_range(req.width, req.height, req.dl, req.dm, req.l_shift, req.m_shift, &lo, &hi);
  const double wrange = req.w_max - req.w_min;
  // w-gridding is skipped only when the whole w spread changes the phase of
  // any pixel by a negligible fraction of epsilon.
  const bool use_w = M_PI * wrange * (hi - lo) > 1e-3 * req.epsilon;
  const double ndim = use_w ? 3.0 : 2.0;
  const double n_vis = std::max<double>(1.0, (double)req.n_vis);
  *fallback = nullptr;
  *fallback_err = std::numeric_limits<double>::infinity();
  std::vector<wgpu_plan_t> out;
  for (int i = 0; i < kEsKernelTableSize; ++i) {
    const EsKernelEntry &e = kEsKernelTable[i];
    if (e.sigma < smin - 1e-9 || e.sigma > smax + 1e-9) continue;
    if (req.force_support > 0 && e.support != req.force_support) continue;
    if (req.force_sigma > 0 && std::fabs(e.sigma - req.force_sigma) > 1e-6) continue;
    // Aliasing: worst case over the image band (a few point sources near the
    // edge see the maximum, not the RMS, error), summed in quadrature over the
    // gridded dimensions.  FP32 round-off: the grid and FFT carry white noise
    // of relative size ~kFp32Noise, which the grid correction magnifies by
    // amp_rms in every corrected dimension.
    const double alias = std::sqrt(ndim) * e.err_max;
    const double fp32 = kFp32Noise * std::pow(e.amp_rms, ndim);
    const double est = std::sqrt(alias * alias + fp32 * fp32);

    wgpu_plan_t p;
    std::memset(&p, 0, sizeof(p));
    p.width = req.width;
    p.height = req.height;
    p.support = e.support;
    p.sigma = e.sigma;
    p.beta = e.beta;
    // uv tiles of 16 x 16 cells: the gridding kernels give one thread to each
    // tile cell and pair a tile with 16 w planes
    const int64_t tile = 16;
    if (req.force_tile > 0 && req.force_tile != tile) continue;
    // row length: the next size with a row-transform schedule
    int64_t nu = good_fft_size((int64_t)std::ceil(e.sigma * req.width), tile);
    while (nu <= fft_row_max_length() && !fft_row_length_supported((int)nu))
      nu = good_fft_size(nu + 1, tile);
    const int64_t nv = good_fft_size((int64_t)std::ceil(e.sigma * req.height), tile);
    if (e.support > tile) continue;
    int64_t f1, f2;
    if (nu > fft_row_max_length() || !try_decompose(nv, &f1, &f2)) continue;
    // the most accurate entry whose grid the transforms take: the plan used
    // when no entry meets epsilon
    if (est < *fallback_err) {
      *fallback_err = est;
      *fallback = &e;
    }
    if (est > req.epsilon) continue;
    p.tile = tile;
    p.nu = nu;
    p.nv = nv;
    p.dl = req.dl;
    p.dm = req.dm;
    p.l_shift = req.l_shift;
    p.m_shift = req.m_shift;
    p.nm1_min = lo;
    p.nm1_max = hi;
    p.nm1_center = 0.5 * (lo + hi);
    if (use_w) {
      p.dw = 1.0 / (e.sigma * (hi - lo));
      p.n_planes = (int64_t)std::ceil(wrange / p.dw) + e.support;
      p.w0 = req.w_min - 0.5 * (double)e.support * p.dw;
    } else {
      p.dw = 1.0;
      p.n_planes = 1;
      p.w0 = 0.5 * (req.w_min + req.w_max);
    }
    p.est_error = est;
    const int64_t rstride = (req.width + 31) / 32 * 32;
    const double w_planes_per_vis = use_w ? (double)e.support : 1.0;
    const double t_grid = 2.0 * n_vis * e.support * e.support * w_planes_per_vis / kCellRate *
                          (e.support > 8 ? kWideSupportFactor : 1.0);
    const double t_fft = 2.0 * (double)p.n_planes *
                         (16.0 * nu * nv + 40.0 * nv * rstride) / kByteRate;
    p.est_seconds = t_grid + t_fft;
    out.push_back(p);
  }
  return out;
}

// Planes resident per pipeline step, and the column decomposition.
void finish_plan(wgpu_plan_t &p, const wgpu_plan_request_t &req) {
  const int64_t rstride = (p.width + 31) / 32 * 32;
  // plane + cropped rows + the gridding units' spilled border cells (at most
  // (W - 1)(2T + W - 1) cells per T x T tile)
  const double spill = (double)(p.support - 1) * (2.0 * p.tile + p.support - 1) /
                       ((double)p.tile * p.tile);
  const double per_plane = 8.0 * p.nu * p.nv * (1.0 + spill) + 8.0 * p.nv * rstride;
  const double budget = req.memory_budget_bytes > 0 ? req.memory_budget_bytes : 64e9;
  int64_t batch = (int64_t)std::floor(budget / per_plane);
  int64_t cap = req.max_plane_batch > 0 ? req.max_plane_batch : 32;
  batch = std::max<int64_t>(1, std::min<int64_t>(std::min(batch, cap), p.n_planes));
  // whole 16-plane gridding groups where the batch allows it
  const int64_t group = grid_plane_group();
  if (batch > group && batch < p.n_planes) batch -= batch % group;
  p.plane_batch = batch;
  fft_decompose(p.nv, &p.fft_n1, &p.fft_n2);
}

}  // namespace

wgpu_plan_t make_plan(const wgpu_plan_request_t &req) {
  check_request(req);
  const EsKernelEntry *fallback;
  double fallback_err;
  const std::vector<wgpu_plan_t> c = feasible_plans(req, &fallback, &fallback_err);
  if (c.empty()) {
    if (fallback == nullptr || req.force_support > 0)
      throw Error(WGPU_ERR_INVALID, "no kernel configuration satisfies the request");
    // Most accurate entry available: retry pinned to it.
    wgpu_plan_request_t r2 = req;
    r2.force_support = fallback->support;
    r2.force_sigma = fallback->sigma;
    r2.epsilon = std::max(req.epsilon, fallback_err * 1.0001);
    return make_plan(r2);
  }
  // lowest cost-model time; the first in table order on ties
  size_t best = 0;
  for (size_t i = 1; i < c.size(); ++i)
    if (c[i].est_seconds < c[best].est_seconds) best = i;
  wgpu_plan_t p = c[best];
  finish_plan(p, req);
  return p;
}

std::vector<wgpu_plan_t> plan_candidates(const wgpu_plan_request_t &req, size_t max_plans) {
  const wgpu_plan_t first = make_plan(req);  // validates; handles the fallback
  const EsKernelEntry *fallback;
  double fallback_err;
  std::vector<wgpu_plan_t> c = feasible_plans(req, &fallback, &fallback_err);
  if (c.empty()) return {first};
  std::stable_sort(c.begin(), c.end(), [](const wgpu_plan_t &a, const wgpu_plan_t &b) {
    return a.est_seconds < b.est_seconds;
  });
  if (c.size() > max_plans) c.resize(std::max<size_t>(1, max_plans));
  for (wgpu_plan_t &p : c) finish_plan(p, req);
  return c;
}

DevPlan to_dev_plan(const wgpu_plan_t &p) {
  DevPlan d;
  d.nu = (int)p.nu;
  d.nv = (int)p.nv;
  d.width = (int)p.width;
  d.height = (int)p.height;
  d.support = (int)p.support;
  d.tile = (int)p.tile;
  d.ntu = (int)(p.nu / p.tile);
  d.ntv = (int)(p.nv / p.tile);
  d.n_planes = (int)p.n_planes;
  d.beta = (float)p.beta;
  d.dl = p.dl;
  d.dm = p.dm;
  d.l_shift = p.l_shift;
  d.m_shift = p.m_shift;
  d.w0 = p.w0;
  d.dw = p.dw;
  d.inv_dw = p.n_planes > 1 ? 1.0 / p.dw : 0.0;
  d.nm1_center = p.nm1_center;
  d.w0f = (float)d.w0;
  d.inv_dwf = (float)d.inv_dw;
  d.w0l = (float)(d.w0 - (double)d.w0f);
  d.inv_dwl = (float)(d.inv_dw - (double)d.inv_dwf);
  d.nm1_center_f = (float)d.nm1_center;
  d.nm1_center_l = (float)(d.nm1_center - (double)d.nm1_center_f);
  d.l_shift_f = (float)d.l_shift;
  d.l_shift_l = (float)(d.l_shift - (double)d.l_shift_f);
  d.m_shift_f = (float)d.m_shift;
  d.m_shift_l = (float)(d.m_shift - (double)d.m_shift_f);
  return d;
}

}  // namespace wgpu
