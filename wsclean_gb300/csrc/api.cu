// C-ABI implementation: the gridder object and the inversion / prediction
// pipelines (host orchestration of the CUDA kernels on one stream).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <limits>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "wgpu_internal.h"

namespace {

thread_local std::string g_last_error;

int fail(int status, const std::string &msg) {
  g_last_error = msg;
  return status;
}

template <typename F>
int guarded(F &&f) {
  try {
    g_last_error.clear();
    f();
    return WGPU_OK;
  } catch (const wgpu::Error &e) {
    return fail(e.status, e.what());
  } catch (const std::bad_alloc &) {
    return fail(WGPU_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception &e) {
    return fail(WGPU_ERR_INVALID, e.what());
  }
}

}  // namespace

namespace wgpu {
int report_failure(int status, const std::string &msg) { return fail(status, msg); }
void clear_failure() { g_last_error.clear(); }
}  // namespace wgpu

// Stage timer: events recorded on the gridder stream between launches; the
// elapsed time of each interval is charged to the stage that opened it.
struct StageTimer {
  std::vector<cudaEvent_t> pool;
  std::vector<std::string> names;
  size_t used = 0;
  cudaStream_t stream = nullptr;

  void begin(cudaStream_t s) {
    stream = s;
    used = 0;
    names.clear();
  }
  void mark(const char *name) {
    if (used == pool.size()) {
      cudaEvent_t e;
      WGPU_CUDA(cudaEventCreate(&e));
      pool.push_back(e);
    }
    WGPU_CUDA(cudaEventRecord(pool[used++], stream));
    names.push_back(name);
  }
  // Returns totals per stage name (last mark is the end marker).
  struct Stage {
    std::string name;
    double ms;
    int count;
  };
  std::vector<Stage> collect() {
    std::vector<Stage> out;
    if (used < 2) return out;
    WGPU_CUDA(cudaEventSynchronize(pool[used - 1]));
    std::map<std::string, size_t> index;
    for (size_t i = 0; i + 1 < used; ++i) {
      float ms = 0.f;
      WGPU_CUDA(cudaEventElapsedTime(&ms, pool[i], pool[i + 1]));
      auto it = index.find(names[i]);
      if (it == index.end()) {
        index[names[i]] = out.size();
        out.push_back({names[i], 0.0, 0});
        it = index.find(names[i]);
      }
      out[it->second].ms += ms;
      out[it->second].count += 1;
    }
    return out;
  }
  ~StageTimer() {
    for (auto e : pool) cudaEventDestroy(e);
  }
};


// Device-resident state of a bound visibility set (see wgpu_gridder_bind):
// bucketing, work items, buffers and the captured inversion / prediction
// graphs, all owned here so that later unbound calls cannot move them.
struct BoundState {
  wgpu_plan_t plan;
  wgpu::DevPlan dp;
  int64_t n_rows = 0, n_chan = 0, n_out = 0;
  std::vector<void *> owned;
  double *uvw = nullptr, *freq = nullptr, *nu_w = nullptr;
  wgpu::ScreenTable scr;
  uint8_t *mask = nullptr;
  wgpu::VisRecord *geom = nullptr, *work = nullptr;
  uint32_t *perm = nullptr, *offsets = nullptr;
  wgpu::RowOccupancy rows_occ;  // rows the bound set's footprints touch
  float2 *vis_in = nullptr, *vis_out = nullptr, *vacc = nullptr;
  float2 *planes = nullptr, *rows = nullptr, *acc = nullptr;
  float *img_corr = nullptr, *cx = nullptr, *cy = nullptr, *gl = nullptr, *wcorr = nullptr;
  std::vector<wgpu::WorkItems> gitems, ditems;
  cudaGraph_t ginv = nullptr, gpred = nullptr;
  cudaGraphExec_t xinv = nullptr, xpred = nullptr;
  uint64_t inv_kernels = 0, pred_kernels = 0;

  void *alloc(size_t bytes) {
    void *p = nullptr;
    WGPU_CUDA(cudaMalloc(&p, bytes ? bytes : 16));
    owned.push_back(p);
    return p;
  }
  ~BoundState() {
    if (xinv) cudaGraphExecDestroy(xinv);
    if (xpred) cudaGraphExecDestroy(xpred);
    if (ginv) cudaGraphDestroy(ginv);
    if (gpred) cudaGraphDestroy(gpred);
    for (void *p : owned) cudaFree(p);
  }
};

struct wgpu_gridder {
  size_t width, height, width_t, height_t, nthreads, verbosity;
  double dl, dm, l_shift, m_shift, epsilon;
  bool tuning;
  int prec;
  int device = 0;
  cudaStream_t stream = nullptr;
  wgpu::DeviceArena arena;
  wgpu::FftTables *fft = nullptr;
  void *d_img = nullptr;
  enum class Mode { kNone, kInversion, kPrediction } mode = Mode::kNone;
  wgpu_plan_t last_plan;
  bool pinned = false;
  wgpu_plan_t pinned_plan;
  StageTimer timer;
  std::vector<StageTimer::Stage> last_timings;
  std::string corr_key;  // geometry of the correction tables in the arena
  std::string nuw_key;   // geometry (and buffer) of the n - 1 table in the arena
  std::string scr_key;   // plan (and buffer) of the w-screen terms in the arena
  std::string wcorr_key; // plan (and buffers) of the w-correction table in the arena
  std::unique_ptr<BoundState> bound;
  std::vector<wgpu_tuning_trial_t> last_trials;  // candidates timed by the last tuning
  double plane_budget = 0;  // >0 caps the plane-batch bytes of every plan
  unsigned *d_flags = nullptr;  // device: expired bounded waits
  unsigned *h_flags = nullptr;  // pinned host copy, read after each call
  void *stage_buf[2] = {};      // page-locked staging chunks for pageable caller memory
  cudaEvent_t stage_ev[2] = {};
};

namespace wgpu {
namespace {

constexpr int kGlNodes = kCorrGlNodes;

// Ends a pipeline: the device flag word is copied behind the last launch, the
// end event is recorded and waited for, and an expired bounded wait is
// reported as WGPU_ERR_TIMEOUT.
void end_call(wgpu_gridder *g) {
  WGPU_CUDA(cudaMemcpyAsync(g->h_flags, g->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            g->stream));
  g->timer.mark("end");
  g->last_timings = g->timer.collect();
  if (*g->h_flags != 0) {
    *g->h_flags = 0;
    WGPU_CUDA(cudaMemsetAsync(g->d_flags, 0, sizeof(unsigned), g->stream));
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
    throw Error(WGPU_ERR_TIMEOUT, "a bounded device wait expired (bucket sort look-back, row "
                                  "transform prefetch or degridding staging)");
  }
}

size_t image_bytes(const wgpu_gridder *g) {
  return g->width_t * g->height_t * (size_t)g->prec;
}

void ensure_image(wgpu_gridder *g) {
  if (!g->d_img) WGPU_CUDA(cudaMalloc(&g->d_img, image_bytes(g)));
}

// ---- copies between caller host memory and the device ------------------------
// Page-locked caller memory (pinned or registered) and small buffers are
// copied directly.  Pageable memory goes through two page-locked staging
// chunks of the gridder: the device copy of one chunk runs while the host
// copies the next, instead of the driver's slower pageable path.
constexpr size_t kStageChunk = 16ull << 20;
constexpr size_t kDirectCopyMax = 4ull << 20;

bool host_is_pinned(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// WGPU_DEBUG_COPIES=1 reports every host copy (direction, bytes, path) on
// stderr, to tell which caller buffers the driver sees as page-locked.
bool debug_copies() {
  static const bool on = [] {
    const char *e = std::getenv("WGPU_DEBUG_COPIES");
    return e && e[0] == '1';
  }();
  return on;
}

void ensure_staging(wgpu_gridder *g) {
  for (int k = 0; k < 2; ++k) {
    if (!g->stage_buf[k])
      WGPU_CUDA(cudaHostAlloc(&g->stage_buf[k], kStageChunk, cudaHostAllocDefault));
    if (!g->stage_ev[k])
      WGPU_CUDA(cudaEventCreateWithFlags(&g->stage_ev[k], cudaEventDisableTiming));
  }
}

// Host to device on the gridder stream; returns once the caller's memory has
// been read (the device copy may still be running).
void copy_to_device(wgpu_gridder *g, void *d, const void *h, size_t bytes) {
  if (bytes == 0) return;
  if (debug_copies())
    std::fprintf(stderr, "wgpu copy h2d %zu bytes %s\n", bytes,
                 host_is_pinned(h) ? "page-locked" : "pageable");
  if (bytes <= kDirectCopyMax || host_is_pinned(h)) {
    WGPU_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, g->stream));
    return;
  }
  ensure_staging(g);
  int k = 0;
  for (size_t off = 0; off < bytes; off += kStageChunk, k ^= 1) {
    const size_t n = std::min(kStageChunk, bytes - off);
    WGPU_CUDA(cudaEventSynchronize(g->stage_ev[k]));  // the chunk's previous copy is done
    std::memcpy(g->stage_buf[k], (const char *)h + off, n);
    WGPU_CUDA(cudaMemcpyAsync((char *)d + off, g->stage_buf[k], n, cudaMemcpyHostToDevice,
                              g->stream));
    WGPU_CUDA(cudaEventRecord(g->stage_ev[k], g->stream));
  }
}

// Device to host after the work queued on the gridder stream; returns when
// the caller's memory holds the data.
void copy_to_host(wgpu_gridder *g, void *h, const void *d, size_t bytes) {
  if (bytes == 0) return;
  if (debug_copies())
    std::fprintf(stderr, "wgpu copy d2h %zu bytes %s\n", bytes,
                 host_is_pinned(h) ? "page-locked" : "pageable");
  if (bytes <= kDirectCopyMax || host_is_pinned(h)) {
    WGPU_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, g->stream));
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
    return;
  }
  ensure_staging(g);
  const size_t n_chunks = (bytes + kStageChunk - 1) / kStageChunk;
  auto issue = [&](size_t c) {
    const size_t off = c * kStageChunk, n = std::min(kStageChunk, bytes - off);
    WGPU_CUDA(cudaMemcpyAsync(g->stage_buf[c & 1], (const char *)d + off, n,
                              cudaMemcpyDeviceToHost, g->stream));
    WGPU_CUDA(cudaEventRecord(g->stage_ev[c & 1], g->stream));
  };
  issue(0);
  if (n_chunks > 1) issue(1);
  for (size_t c = 0; c < n_chunks; ++c) {
    WGPU_CUDA(cudaEventSynchronize(g->stage_ev[c & 1]));
    const size_t off = c * kStageChunk, n = std::min(kStageChunk, bytes - off);
    std::memcpy((char *)h + off, g->stage_buf[c & 1], n);
    if (c + 2 < n_chunks) issue(c + 2);  // into the chunk just emptied
  }
}

// The caller's float image (width x height) from the gridder's image (trimmed
// width_t x height_t, float or double): NaN outside the trimmed region.
__global__ void image_out_kernel(const void *__restrict__ img, int prec, int64_t wt, int64_t ht,
                                 int64_t w, int64_t h, float *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w * h) return;
  const int64_t x = i % w, y = i / w;
  const int64_t xs = x - (w - wt) / 2, ys = y - (h - ht) / 2;
  float v = __int_as_float(0x7fc00000);  // quiet NaN
  if (xs >= 0 && xs < wt && ys >= 0 && ys < ht) {
    const int64_t j = ys * wt + xs;
    v = prec == 8 ? __double2float_rn(((const double *)img)[j]) : ((const float *)img)[j];
  }
  out[i] = v;
}

// The gridder's image (trimmed region, float or double) from the caller's
// float image.
__global__ void image_in_kernel(const float *__restrict__ in, int prec, int64_t wt, int64_t ht,
                                int64_t w, int64_t h, void *__restrict__ img) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= wt * ht) return;
  const int64_t xs = i % wt, ys = i / wt;
  const float v = in[(xs + (w - wt) / 2) + (ys + (h - ht) / 2) * w];
  if (prec == 8)
    ((double *)img)[i] = (double)v;
  else
    ((float *)img)[i] = v;
}

// Correction tables for one plan, computed on the device: cx, cy (1/psihat per
// column/row) and the quadrature nodes (z_q, w_q phi(z_q)) of the per-pixel w
// factor.
void upload_corrections(wgpu_gridder *g, const wgpu_plan_t &plan, float **cx,
                        float **cy, float **gl) {
  // The tables depend on the kernel and grid geometry only: reuse them while
  // the plan keeps those.
  char key[256];
  std::snprintf(key, sizeof(key), "%.17g/%lld/%lld/%lld/%lld/%lld", plan.beta,
                (long long)plan.support, (long long)plan.nu, (long long)plan.nv,
                (long long)plan.width, (long long)plan.height);
  if (g->corr_key == key) {
    *cx = (float *)g->arena.get(kSlotCorrX, sizeof(float) * plan.width);
    *cy = (float *)g->arena.get(kSlotCorrY, sizeof(float) * plan.height);
    *gl = (float *)g->arena.get(kSlotGl, sizeof(float) * 2 * kGlNodes);
    return;
  }
  *cx = (float *)g->arena.get(kSlotCorrX, sizeof(float) * plan.width);
  *cy = (float *)g->arena.get(kSlotCorrY, sizeof(float) * plan.height);
  *gl = (float *)g->arena.get(kSlotGl, sizeof(float) * 2 * kGlNodes);
  launch_correction_tables(plan, *cx, *cy, *gl, g->stream);
  g->corr_key = key;
}

// Per-pixel n - 1 - c_n table (FP64) of the plan's image geometry, in the
// arena; recomputed only when that geometry or the buffer changes.
double *nu_table_for(wgpu_gridder *g, const wgpu_plan_t &plan, const DevPlan &dp) {
  double *nu_w = (double *)g->arena.get(kSlotNuW, sizeof(double) * plan.width * plan.height);
  char key[320];
  std::snprintf(key, sizeof(key), "%p/%lld/%lld/%.17g/%.17g/%.17g/%.17g/%.17g", (void *)nu_w,
                (long long)plan.width, (long long)plan.height, plan.dl, plan.dm, plan.l_shift,
                plan.m_shift, plan.nm1_center);
  if (g->nuw_key != key) {
    launch_nu_table(dp, nu_w, g->stream);
    g->nuw_key = key;
  }
  return nu_w;
}

// Per-pixel w-screen terms of the plan (w0, dw and the geometry of nu_w), in
// the arena; recomputed only when the plan's w planes or the buffers change.
ScreenTable screen_table_for(wgpu_gridder *g, const wgpu_plan_t &plan, const DevPlan &dp,
                             const double *nu_w) {
  const int64_t npix = plan.width * plan.height;
  void *buf = g->arena.get(kSlotScreen, kScreenBytesPerPixel * npix);
  char key[400];
  std::snprintf(key, sizeof(key), "%s/%p/%.17g/%.17g", g->nuw_key.c_str(), buf, dp.w0, dp.dw);
  const ScreenTable scr = screen_table_at(buf, npix);
  if (g->scr_key != key) {
    launch_screen_table(dp, nu_w, scr, g->stream);
    g->scr_key = key;
  }
  return scr;
}

// Per-pixel w correction of the plan, in the arena; recomputed only when the
// plan's w planes, kernel or the buffers change.
const float *wcorr_table_for(wgpu_gridder *g, const wgpu_plan_t &plan, const DevPlan &dp,
                             const double *nu_w, const float *gl) {
  float *wc = (float *)g->arena.get(kSlotWCorr, sizeof(float) * plan.width * plan.height);
  char key[480];
  std::snprintf(key, sizeof(key), "%s/%p/%p/%.17g/%.17g/%d/%lld", g->nuw_key.c_str(), (void *)wc,
                (const void *)gl, dp.dw, (double)dp.beta, dp.support, (long long)dp.n_planes);
  if (g->wcorr_key != key) {
    launch_wcorr_table(dp, nu_w, gl, kGlNodes, wc, g->stream);
    g->wcorr_key = key;
  }
  return wc;
}

// A pinned plan is used as long as it covers the data: every visibility's w
// footprint must fall inside its planes (a clamped footprint would be wrong).
void check_pinned_plan(const wgpu_gridder *g, double w_min, double w_max) {
  const wgpu_plan_t &p = g->pinned_plan;
  if (p.width != (int64_t)g->width_t || p.height != (int64_t)g->height_t ||
      p.dl != g->dl || p.dm != g->dm || p.l_shift != g->l_shift || p.m_shift != g->m_shift)
    throw Error(WGPU_ERR_INVALID, "pinned plan does not match the gridder geometry");
  if (p.n_planes > 1) {
    const double half = 0.5 * (double)p.support;
    const double lo = p.w0 + (half - 1.0) * p.dw, hi = p.w0 + ((double)p.n_planes - half) * p.dw;
    if (!(w_min > lo) || !(w_max <= hi))
      throw Error(WGPU_ERR_INVALID, "data w range exceeds the pinned plan's planes");
  } else {
    const double dev = std::max(std::fabs(w_min - p.w0), std::fabs(w_max - p.w0));
    if (M_PI * dev * (p.nm1_max - p.nm1_min) > 1e-3 * g->epsilon)
      throw Error(WGPU_ERR_INVALID, "data w range needs w-planes but the pinned plan has one");
  }
}

wgpu_plan_request_t plan_request(const wgpu_gridder *g, double w_min, double w_max,
                                 int64_t n_vis) {
  wgpu_plan_request_t r;
  std::memset(&r, 0, sizeof(r));
  r.width = (int64_t)g->width_t;
  r.height = (int64_t)g->height_t;
  r.dl = g->dl;
  r.dm = g->dm;
  r.l_shift = g->l_shift;
  r.m_shift = g->m_shift;
  r.epsilon = g->epsilon;
  r.w_min = w_min;
  r.w_max = w_max;
  r.n_vis = n_vis;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
    r.memory_budget_bytes = std::min(64e9, 0.4 * (double)(free_b + g->arena.total()));
  }
  if (g->plane_budget > 0) r.memory_budget_bytes = g->plane_budget;
  // WGPU_PLANE_BUDGET_GB caps the plane-batch memory (profiling small cases)
  if (const char *env = std::getenv("WGPU_PLANE_BUDGET_GB")) {
    const double gb = std::atof(env);
    if (gb > 0) r.memory_budget_bytes = gb * 1e9;
  }
  return r;
}

wgpu_plan_t plan_for(wgpu_gridder *g, double w_min, double w_max, int64_t n_vis) {
  if (g->pinned) {
    check_pinned_plan(g, w_min, w_max);
    return g->pinned_plan;
  }
  return make_plan(plan_request(g, w_min, w_max, n_vis));
}

// ---- autotuning: candidate plans timed on the caller's own samples ----------
// The reference's `tuning` flag selects ducc0's tuned entry points
// (wgridder/gridder_simple.h:216-225, gridder_simple_implementation.h:185-194),
// whose internals are not part of the reference tree.  Here the flag makes the
// plan a measured choice: the cost model ranks the (support, sigma) entries
// that meet epsilon, and the best kTuneCandidates of them are run on the
// call's own samples on this device (bucketing, then every plane batch's
// gridding and forward FFT passes, or backward FFT passes and degridding),
// timed with events on the gridder's stream.  The fastest is used.  The choice
// is remembered per device and request shape: image geometry, epsilon,
// direction, the sample count to within a factor of sqrt(2) and the w range to
// within 2^(1/4).  Later calls of that shape, including those of new gridders
// (WSClean creates one per major cycle), plan without timing.  The uv tile is
// not a tuning dimension: the gridding kernels give one thread to each of its
// 16 x 16 cells.
constexpr size_t kTuneCandidates = 3;

struct TuneChoice {
  int64_t support;
  double sigma;
};
std::mutex g_tune_mu;
std::map<std::string, TuneChoice> g_tune_cache;

std::string tune_key(const wgpu_gridder *g, char direction, double w_min, double w_max,
                     int64_t n_vis) {
  const double wr = w_max - w_min;
  char buf[384];
  std::snprintf(buf, sizeof(buf), "%d|%c|%zu|%zu|%.17g|%.17g|%.17g|%.17g|%.17g|%.17g|%d|%d",
                g->device, direction, g->width_t, g->height_t, g->dl, g->dm, g->l_shift,
                g->m_shift, g->epsilon, g->plane_budget,
                (int)std::floor(2.0 * std::log2((double)std::max<int64_t>(n_vis, 1))),
                wr > 0 ? (int)std::floor(4.0 * std::log2(wr)) : -100000);
  return buf;
}

// Device time of one plan on the given samples: the bucketing, then every
// plane batch of the inversion (gridding, forward FFT passes into a scratch
// accumulator) and/or of the prediction (backward FFT passes of a zero image,
// degridding into scratch sums).  Nothing the gridder keeps is written.  A
// short run is repeated (up to three times) and the least time kept, so that
// first-launch costs do not decide between small plans.
double time_plan(wgpu_gridder *g, const wgpu_plan_t &plan, const double *d_uvw,
                 const double *d_freq, const float *d_vis, const uint8_t *d_mask,
                 size_t n_rows, size_t n_chan, bool skip_zero, bool inversion,
                 bool prediction) {
  cudaStream_t s = g->stream;
  const DevPlan dp = to_dev_plan(plan);
  const int64_t npix = plan.width * plan.height;
  const int rstride = (int)((plan.width + 31) / 32 * 32);
  const int64_t B = plan.plane_batch;
  // tables outside the timed region (their creation copies synchronously)
  fft_twiddles(*g->fft, (int)plan.nu);
  fft_twiddles(*g->fft, (int)plan.nv);
  fft_twiddles(*g->fft, (int)plan.fft_n1);
  fft_twiddles(*g->fft, (int)plan.fft_n2);
  fft_prepare_rows(*g->fft, (int)plan.nu);
  const ScreenTable scr = screen_table_for(g, plan, dp, nu_table_for(g, plan, dp));
  float2 *planes = (float2 *)g->arena.get(kSlotPlanes, sizeof(float2) * B * plan.nu * plan.nv);
  float2 *R = (float2 *)g->arena.get(kSlotRows, sizeof(float2) * B * plan.nv * rstride);
  float2 *acc = inversion ? (float2 *)g->arena.get(kSlotAcc, sizeof(float2) * npix) : nullptr;
  float *img = prediction ? (float *)g->arena.get(kSlotImgCorr, sizeof(float) * npix) : nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  WGPU_CUDA(cudaEventCreate(&e0));
  WGPU_CUDA(cudaEventCreate(&e1));
  double best = std::numeric_limits<double>::infinity();
  try {
    for (int rep = 0; rep < 3; ++rep) {
      WGPU_CUDA(cudaStreamSynchronize(s));
      WGPU_CUDA(cudaEventRecord(e0, s));
      const BucketResult b = bucket_visibilities(g->arena, dp, d_uvw, d_freq, d_vis, d_mask,
                                                 (int64_t)n_rows, (int64_t)n_chan, skip_zero,
                                                 g->d_flags, s);
      if (inversion) {
        WGPU_CUDA(cudaMemsetAsync(acc, 0, sizeof(float2) * npix, s));
        for (int64_t p0 = 0; p0 < plan.n_planes; p0 += B) {
          const int nb = (int)std::min<int64_t>(B, plan.n_planes - p0);
          const RowSel sel = row_sel(b.rows, (int)p0);
          launch_grid(g->arena, dp, b.records, b.offsets, (int)p0, nb, planes, s);
          launch_fft_rows_forward_crop(*g->fft, dp, planes, R, rstride, nb, sel, g->d_flags, s);
          launch_fft_cols_a(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2, R, rstride, nb,
                            -1.0f, sel, s);
          launch_fft_cols_b_forward_accumulate(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2,
                                               R, rstride, nb, (int)p0, scr, acc, sel, s);
        }
      }
      if (prediction) {
        float2 *vacc = (float2 *)g->arena.get(kSlotVisAcc, sizeof(float2) * (b.n_out + 1));
        WGPU_CUDA(cudaMemsetAsync(img, 0, sizeof(float) * npix, s));
        WGPU_CUDA(cudaMemsetAsync(vacc, 0, sizeof(float2) * (b.n_out + 1), s));
        for (int64_t p0 = 0; p0 < plan.n_planes; p0 += B) {
          const int nb = (int)std::min<int64_t>(B, plan.n_planes - p0);
          const RowSel sel = row_sel(b.rows, (int)p0);
          launch_fft_cols_b_backward_screen(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2,
                                            img, scr, R, rstride, nb, (int)p0, s);
          launch_fft_cols_a(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2, R, rstride, nb,
                            +1.0f, sel, s);
          launch_fft_rows_backward_pad(*g->fft, dp, R, rstride, planes, nb, sel, g->d_flags, s);
          launch_degrid(g->arena, dp, b.records, b.offsets, (int)p0, nb, planes, vacc,
                        g->d_flags, s);
        }
      }
      WGPU_CUDA(cudaEventRecord(e1, s));
      WGPU_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      WGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best = std::min(best, (double)ms);
      if (ms > 20.f) break;
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

}  // namespace

void tuning_cache_clear() {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache.clear();
}

namespace {

// The plan for a call of a tuning gridder (see above).  `run` times one
// candidate plan.  A shape seen before takes its remembered choice when that
// entry still meets the request; the trials of the last tuning are kept in
// the gridder.
wgpu_plan_t tuned_plan(wgpu_gridder *g, char direction, double w_min, double w_max,
                       int64_t n_vis, const std::function<double(const wgpu_plan_t &)> &run) {
  g->last_trials.clear();
  if (g->pinned) return plan_for(g, w_min, w_max, n_vis);
  const wgpu_plan_request_t r = plan_request(g, w_min, w_max, n_vis);
  const std::vector<wgpu_plan_t> all = plan_candidates(r, 1000);
  const std::string key = tune_key(g, direction, w_min, w_max, n_vis);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end())
      for (const wgpu_plan_t &p : all)
        if (p.support == it->second.support && p.sigma == it->second.sigma) return p;
  }
  std::vector<wgpu_plan_t> cands(all.begin(),
                                 all.begin() + std::min(all.size(), kTuneCandidates));
  size_t best = 0;
  if (cands.size() > 1) {
    // A candidate whose buffers do not fit in the device memory left is
    // skipped (its time counts as infinite); the first, untuned plan is the
    // one that must run.
    auto timed = [&](const wgpu_plan_t &c, bool required) -> double {
      try {
        return run(c);
      } catch (const Error &e) {
        if (e.status != WGPU_ERR_NOMEM || required) throw;
        return std::numeric_limits<double>::infinity();
      }
    };
    // one untimed run of the plan with the largest buffers first, so that the
    // arena's allocations are not charged to whichever candidate runs first
    size_t big = 0;
    for (size_t i = 1; i < cands.size(); ++i)
      if (cands[i].n_planes * cands[i].nu * cands[i].nv >
          cands[big].n_planes * cands[big].nu * cands[big].nv)
        big = i;
    timed(cands[big], false);
    std::vector<double> ms(cands.size());
    for (size_t i = 0; i < cands.size(); ++i) {
      ms[i] = timed(cands[i], i == 0);
      if (ms[i] < ms[best]) best = i;
    }
    for (size_t i = 0; i < cands.size(); ++i) {
      wgpu_tuning_trial_t t;
      std::memset(&t, 0, sizeof(t));
      t.support = cands[i].support;
      t.sigma = cands[i].sigma;
      t.nu = cands[i].nu;
      t.nv = cands[i].nv;
      t.n_planes = cands[i].n_planes;
      t.est_seconds = cands[i].est_seconds;
      t.measured_ms = ms[i];
      t.chosen = i == best ? 1 : 0;
      g->last_trials.push_back(t);
    }
    if (g->verbosity > 0)
      for (const wgpu_tuning_trial_t &t : g->last_trials)
        std::fprintf(stderr, "wgpu tuning: W=%lld sigma=%.2f grid %lld planes %lld: %.2f ms%s\n",
                     (long long)t.support, t.sigma, (long long)t.nu, (long long)t.n_planes,
                     t.measured_ms, t.chosen ? " (chosen)" : "");
  }
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[key] = TuneChoice{cands[best].support, cands[best].sigma};
  }
  return cands[best];
}

void log_plan(const wgpu_gridder *g, const char *what, const wgpu_plan_t &p,
              int64_t n_vis) {
  if (g->verbosity == 0) return;
  std::fprintf(stderr,
               "wgpu %s: %lld vis, image %lldx%lld, grid %lldx%lld, W=%lld sigma=%.2f "
               "beta=%.3f planes=%lld (batch %lld) est.err=%.2e\n",
               what, (long long)n_vis, (long long)p.width, (long long)p.height,
               (long long)p.nu, (long long)p.nv, (long long)p.support, p.sigma,
               p.beta, (long long)p.n_planes, (long long)p.plane_batch,
               p.est_error);
}

void invert_device(wgpu_gridder *g, size_t n_rows, size_t n_chan,
                   const double *d_uvw, const double *d_freq, const float *d_vis) {
  if (g->mode != wgpu_gridder::Mode::kInversion)
    throw Error(WGPU_ERR_STATE, "AddInversionData before InitializeInversion");
  if (n_rows == 0 || n_chan == 0) return;
  cudaStream_t s = g->stream;
  g->timer.begin(s);
  g->timer.mark("extent");
  double w_min, w_max;
  int64_t count;
  compute_w_extent(d_uvw, d_freq, d_vis, nullptr, (int64_t)n_rows, (int64_t)n_chan, true,
                   &w_min, &w_max, &count,
                   g->arena.get(kSlotErr, w_extent_scratch_bytes((int64_t)n_chan)), s);
  if (count == 0) {
    end_call(g);
    return;
  }
  g->timer.mark("tune");
  const wgpu_plan_t plan =
      g->tuning ? tuned_plan(g, 'i', w_min, w_max, count,
                             [&](const wgpu_plan_t &c) {
                               return time_plan(g, c, d_uvw, d_freq, d_vis, nullptr, n_rows,
                                                n_chan, true, true, false);
                             })
                : plan_for(g, w_min, w_max, count);
  g->last_plan = plan;
  log_plan(g, "invert", plan, count);
  const DevPlan dp = to_dev_plan(plan);
  g->timer.mark("bucket");
  const BucketResult b = bucket_visibilities(g->arena, dp, d_uvw, d_freq, d_vis, nullptr,
                                             (int64_t)n_rows, (int64_t)n_chan, true, g->d_flags,
                                             s);
  g->timer.mark("setup");
  const int64_t npix = plan.width * plan.height;
  const int rstride = (int)((plan.width + 31) / 32 * 32);
  double *nu_w = nu_table_for(g, plan, dp);
  const ScreenTable scr = screen_table_for(g, plan, dp, nu_w);
  float2 *acc = (float2 *)g->arena.get(kSlotAcc, sizeof(float2) * npix);
  const int64_t B = plan.plane_batch;
  float2 *planes = (float2 *)g->arena.get(kSlotPlanes, sizeof(float2) * B * plan.nu * plan.nv);
  float2 *R = (float2 *)g->arena.get(kSlotRows, sizeof(float2) * B * plan.nv * rstride);
  WGPU_CUDA(cudaMemsetAsync(acc, 0, sizeof(float2) * npix, s));
  for (int64_t p0 = 0; p0 < plan.n_planes; p0 += B) {
    const int nb = (int)std::min<int64_t>(B, plan.n_planes - p0);
    g->timer.mark("grid");
    launch_grid(g->arena, dp, b.records, b.offsets, (int)p0, nb, planes, s);
    g->timer.mark("fft_rows");
    const RowSel sel = row_sel(b.rows, (int)p0);
    launch_fft_rows_forward_crop(*g->fft, dp, planes, R, rstride, nb, sel, g->d_flags, s);
    g->timer.mark("fft_cols_a");
    launch_fft_cols_a(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2, R, rstride, nb, -1.0f,
                      sel, s);
    g->timer.mark("fft_cols_b_screen");
    launch_fft_cols_b_forward_accumulate(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2, R,
                                         rstride, nb, (int)p0, scr, acc, sel, s);
    if (g->verbosity >= 2)
      std::fprintf(stderr, "wgpu invert: planes %lld..%lld\n", (long long)p0,
                   (long long)(p0 + nb - 1));
  }
  g->timer.mark("finalize");
  float *cx, *cy, *gl;
  upload_corrections(g, plan, &cx, &cy, &gl);
  launch_finalize_add(dp, acc, wcorr_table_for(g, plan, dp, nu_w, gl), cx, cy, g->d_img, g->prec,
                      s);
  end_call(g);
}

void predict_device(wgpu_gridder *g, size_t n_rows, size_t n_chan,
                    const double *d_uvw, const double *d_freq,
                    const uint8_t *d_mask, float *d_vis) {
  if (g->mode != wgpu_gridder::Mode::kPrediction)
    throw Error(WGPU_ERR_STATE, "PredictVisibilities before InitializePrediction");
  if (n_rows == 0 || n_chan == 0) return;
  cudaStream_t s = g->stream;
  g->timer.begin(s);
  g->timer.mark("extent");
  double w_min, w_max;
  int64_t count;
  compute_w_extent(d_uvw, d_freq, nullptr, d_mask, (int64_t)n_rows, (int64_t)n_chan, false,
                   &w_min, &w_max, &count,
                   g->arena.get(kSlotErr, w_extent_scratch_bytes((int64_t)n_chan)), s);
  if (d_mask) {
    WGPU_CUDA(cudaMemsetAsync(d_vis, 0, sizeof(float2) * n_rows * n_chan, s));
    if (count == 0) {
      end_call(g);
      return;
    }
  }
  g->timer.mark("tune");
  const wgpu_plan_t plan =
      g->tuning ? tuned_plan(g, 'p', w_min, w_max, count,
                             [&](const wgpu_plan_t &c) {
                               return time_plan(g, c, d_uvw, d_freq, nullptr, d_mask, n_rows,
                                                n_chan, false, false, true);
                             })
                : plan_for(g, w_min, w_max, count);
  g->last_plan = plan;
  log_plan(g, "predict", plan, count);
  const DevPlan dp = to_dev_plan(plan);
  g->timer.mark("bucket");
  const BucketResult b = bucket_visibilities(g->arena, dp, d_uvw, d_freq, nullptr, d_mask,
                                             (int64_t)n_rows, (int64_t)n_chan, false, g->d_flags,
                                             s);
  g->timer.mark("setup");
  const int64_t npix = plan.width * plan.height;
  const int rstride = (int)((plan.width + 31) / 32 * 32);
  double *nu_w = nu_table_for(g, plan, dp);
  const ScreenTable scr = screen_table_for(g, plan, dp, nu_w);
  float *img_corr = (float *)g->arena.get(kSlotImgCorr, sizeof(float) * npix);
  float2 *vacc = (float2 *)g->arena.get(kSlotVisAcc, sizeof(float2) * (b.n_out + 1));
  const int64_t B = plan.plane_batch;
  float2 *planes = (float2 *)g->arena.get(kSlotPlanes, sizeof(float2) * B * plan.nu * plan.nv);
  float2 *R = (float2 *)g->arena.get(kSlotRows, sizeof(float2) * B * plan.nv * rstride);
  float *cx, *cy, *gl;
  upload_corrections(g, plan, &cx, &cy, &gl);
  launch_precorrect(dp, g->d_img, g->prec, wcorr_table_for(g, plan, dp, nu_w, gl), cx, cy,
                    img_corr, s);
  WGPU_CUDA(cudaMemsetAsync(vacc, 0, sizeof(float2) * (b.n_out + 1), s));
  for (int64_t p0 = 0; p0 < plan.n_planes; p0 += B) {
    const int nb = (int)std::min<int64_t>(B, plan.n_planes - p0);
    g->timer.mark("fft_cols_b_screen");
    launch_fft_cols_b_backward_screen(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2,
                                      img_corr, scr, R, rstride, nb, (int)p0, s);
    g->timer.mark("fft_cols_a");
    const RowSel sel = row_sel(b.rows, (int)p0);
    launch_fft_cols_a(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2, R, rstride, nb, +1.0f,
                      sel, s);
    g->timer.mark("fft_rows");
    launch_fft_rows_backward_pad(*g->fft, dp, R, rstride, planes, nb, sel, g->d_flags, s);
    g->timer.mark("degrid");
    launch_degrid(g->arena, dp, b.records, b.offsets, (int)p0, nb, planes, vacc, g->d_flags, s);
  }
  g->timer.mark("finalize");
  launch_unpermute_predict(b.perm, vacc, b.n_out, (float2 *)d_vis, s);
  end_call(g);
}

// ---- bound visibility sets: plan and bucket once, replay captured graphs ----

void bind_visibilities(wgpu_gridder *g, size_t n_rows, size_t n_chan, const double *h_uvw,
                       const double *h_freq, const uint8_t *h_mask) {
  g->bound.reset();
  if (n_rows == 0 || n_chan == 0) throw Error(WGPU_ERR_INVALID, "empty visibility set");
  cudaStream_t s = g->stream;
  ensure_image(g);
  auto b = std::make_unique<BoundState>();
  const int64_t n = (int64_t)(n_rows * n_chan);
  b->n_rows = (int64_t)n_rows;
  b->n_chan = (int64_t)n_chan;
  b->uvw = (double *)b->alloc(sizeof(double) * 3 * n_rows);
  b->freq = (double *)b->alloc(sizeof(double) * n_chan);
  copy_to_device(g, b->uvw, h_uvw, sizeof(double) * 3 * n_rows);
  copy_to_device(g, b->freq, h_freq, sizeof(double) * n_chan);
  if (h_mask) {
    b->mask = (uint8_t *)b->alloc((size_t)n);
    copy_to_device(g, b->mask, h_mask, (size_t)n);
  }
  double w_min, w_max;
  int64_t count;
  compute_w_extent(b->uvw, b->freq, nullptr, b->mask, b->n_rows, b->n_chan, false, &w_min,
                   &w_max, &count, g->arena.get(kSlotErr, w_extent_scratch_bytes(b->n_chan)), s);
  if (count == 0) throw Error(WGPU_ERR_INVALID, "the mask selects no visibility");
  BoundState *bs = b.get();
  b->plan = g->tuning ? tuned_plan(g, 'b', w_min, w_max, count,
                                   [&](const wgpu_plan_t &c) {
                                     return time_plan(g, c, bs->uvw, bs->freq, nullptr, bs->mask,
                                                      n_rows, n_chan, false, true, true);
                                   })
                      : plan_for(g, w_min, w_max, count);
  if (g->tuning) {
    // the bound set owns its batch buffers: drop the ones the timing runs used
    for (int slot : {kSlotPlanes, kSlotRows, kSlotAcc, kSlotImgCorr, kSlotVisAcc, kSlotScreen,
                     kSlotWCorr})
      g->arena.release(slot);
    g->scr_key.clear();
    g->wcorr_key.clear();
  }
  g->last_plan = b->plan;
  log_plan(g, "bind", b->plan, count);
  const wgpu_plan_t &plan = b->plan;
  b->dp = to_dev_plan(plan);
  const DevPlan &dp = b->dp;
  const BucketResult br = bucket_visibilities(g->arena, dp, b->uvw, b->freq, nullptr, b->mask,
                                              b->n_rows, b->n_chan, false, g->d_flags, s);
  b->n_out = br.n_out;
  b->geom = (VisRecord *)b->alloc(sizeof(VisRecord) * (br.n_out + 1));
  b->work = (VisRecord *)b->alloc(sizeof(VisRecord) * (br.n_out + 1));
  b->perm = (uint32_t *)b->alloc(sizeof(uint32_t) * (br.n_out + 1));
  b->offsets = (uint32_t *)b->alloc(sizeof(uint32_t) * (br.n_keys + 1));
  WGPU_CUDA(cudaMemcpyAsync(b->geom, br.records, sizeof(VisRecord) * br.n_out,
                            cudaMemcpyDeviceToDevice, s));
  WGPU_CUDA(cudaMemcpyAsync(b->perm, br.perm, sizeof(uint32_t) * br.n_out,
                            cudaMemcpyDeviceToDevice, s));
  WGPU_CUDA(cudaMemcpyAsync(b->offsets, br.offsets, sizeof(uint32_t) * (br.n_keys + 1),
                            cudaMemcpyDeviceToDevice, s));
  b->rows_occ = copy_row_occupancy(br.rows, b->alloc(br.rows.bytes()), s);
  const int64_t npix = plan.width * plan.height;
  const int rstride = (int)((plan.width + 31) / 32 * 32);
  const int64_t B = plan.plane_batch;
  b->vis_in = (float2 *)b->alloc(sizeof(float2) * n);
  b->vis_out = (float2 *)b->alloc(sizeof(float2) * n);
  b->vacc = (float2 *)b->alloc(sizeof(float2) * (br.n_out + 1));
  b->planes = (float2 *)b->alloc(sizeof(float2) * B * plan.nu * plan.nv);
  b->rows = (float2 *)b->alloc(sizeof(float2) * B * plan.nv * rstride);
  b->acc = (float2 *)b->alloc(sizeof(float2) * npix);
  b->nu_w = (double *)b->alloc(sizeof(double) * npix);
  b->scr = screen_table_at(b->alloc(kScreenBytesPerPixel * npix), npix);
  b->img_corr = (float *)b->alloc(sizeof(float) * npix);
  b->cx = (float *)b->alloc(sizeof(float) * plan.width);
  b->cy = (float *)b->alloc(sizeof(float) * plan.height);
  b->gl = (float *)b->alloc(sizeof(float) * 2 * kGlNodes);
  launch_nu_table(dp, b->nu_w, s);
  launch_screen_table(dp, b->nu_w, b->scr, s);
  float *cx, *cy, *gl;
  upload_corrections(g, plan, &cx, &cy, &gl);
  WGPU_CUDA(cudaMemcpyAsync(b->cx, cx, sizeof(float) * plan.width, cudaMemcpyDeviceToDevice, s));
  WGPU_CUDA(cudaMemcpyAsync(b->cy, cy, sizeof(float) * plan.height, cudaMemcpyDeviceToDevice, s));
  WGPU_CUDA(cudaMemcpyAsync(b->gl, gl, sizeof(float) * 2 * kGlNodes, cudaMemcpyDeviceToDevice, s));
  b->wcorr = (float *)b->alloc(sizeof(float) * npix);
  launch_wcorr_table(dp, b->nu_w, b->gl, kGlNodes, b->wcorr, s);
  // twiddle tables are created outside the capture (they are copied synchronously)
  fft_twiddles(*g->fft, (int)plan.nu);
  fft_twiddles(*g->fft, (int)plan.nv);
  fft_twiddles(*g->fft, (int)plan.fft_n1);
  fft_twiddles(*g->fft, (int)plan.fft_n2);
  fft_prepare_rows(*g->fft, (int)plan.nu);
  BoundState *bp = b.get();
  const ItemAlloc own = [bp](int, size_t bytes) -> void * { return bp->alloc(bytes); };
  for (int64_t p0 = 0; p0 < plan.n_planes; p0 += B) {
    const int nb = (int)std::min<int64_t>(B, plan.n_planes - p0);
    b->gitems.push_back(plan_grid_items(dp, b->offsets, (int)p0, nb, own, s));
    b->ditems.push_back(plan_degrid_items(dp, b->offsets, (int)p0, nb, own, s));
  }
  WGPU_CUDA(cudaStreamSynchronize(s));

  // inversion graph: records from the new visibilities, then the batches
  uint64_t k0 = thread_launch_count();
  WGPU_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  try {
    launch_restamp(b->geom, b->perm, b->vis_in, b->n_out, b->work, s);
    WGPU_CUDA(cudaMemsetAsync(b->acc, 0, sizeof(float2) * npix, s));
    for (size_t i = 0; i < b->gitems.size(); ++i) {
      const int p0 = (int)(i * B);
      const int nb = (int)std::min<int64_t>(B, plan.n_planes - p0);
      launch_zero_split_units(dp, b->gitems[i], p0, nb, b->planes, s);
      launch_grid_items(dp, b->work, b->offsets, p0, nb, b->gitems[i], b->planes, s);
      const RowSel sel = row_sel(b->rows_occ, p0);
      launch_fft_rows_forward_crop(*g->fft, dp, b->planes, b->rows, rstride, nb, sel, g->d_flags,
                                   s);
      launch_fft_cols_a(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2, b->rows, rstride, nb,
                        -1.0f, sel, s);
      launch_fft_cols_b_forward_accumulate(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2,
                                           b->rows, rstride, nb, p0, b->scr, b->acc, sel, s);
    }
    launch_finalize_add(dp, b->acc, b->wcorr, b->cx, b->cy, g->d_img, g->prec, s);
  } catch (...) {
    cudaGraph_t junk;
    cudaStreamEndCapture(s, &junk);
    if (junk) cudaGraphDestroy(junk);
    throw;
  }
  WGPU_CUDA(cudaStreamEndCapture(s, &b->ginv));
  WGPU_CUDA(cudaGraphInstantiate(&b->xinv, b->ginv, 0));
  b->inv_kernels = thread_launch_count() - k0;
  count_launch(-(int)b->inv_kernels);  // captured, not run

  // prediction graph: pre-correction, the batches, un-permute
  k0 = thread_launch_count();
  WGPU_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  try {
    launch_precorrect(dp, g->d_img, g->prec, b->wcorr, b->cx, b->cy, b->img_corr, s);
    WGPU_CUDA(cudaMemsetAsync(b->vacc, 0, sizeof(float2) * (b->n_out + 1), s));
    for (size_t i = 0; i < b->ditems.size(); ++i) {
      const int p0 = (int)(i * B);
      const int nb = (int)std::min<int64_t>(B, plan.n_planes - p0);
      launch_fft_cols_b_backward_screen(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2,
                                        b->img_corr, b->scr, b->rows, rstride, nb, p0, s);
      const RowSel sel = row_sel(b->rows_occ, p0);
      launch_fft_cols_a(*g->fft, dp, (int)plan.fft_n1, (int)plan.fft_n2, b->rows, rstride, nb,
                        +1.0f, sel, s);
      launch_fft_rows_backward_pad(*g->fft, dp, b->rows, rstride, b->planes, nb, sel, g->d_flags,
                                   s);
      launch_degrid_items(dp, b->geom, b->offsets, p0, nb, b->ditems[i], b->planes, b->vacc,
                          g->d_flags, s);
    }
    WGPU_CUDA(cudaMemsetAsync(b->vis_out, 0, sizeof(float2) * n, s));
    launch_unpermute_predict(b->perm, b->vacc, b->n_out, b->vis_out, s);
  } catch (...) {
    cudaGraph_t junk;
    cudaStreamEndCapture(s, &junk);
    if (junk) cudaGraphDestroy(junk);
    throw;
  }
  WGPU_CUDA(cudaStreamEndCapture(s, &b->gpred));
  WGPU_CUDA(cudaGraphInstantiate(&b->xpred, b->gpred, 0));
  b->pred_kernels = thread_launch_count() - k0;
  count_launch(-(int)b->pred_kernels);
  // the bucketing's bounded waits report into the flag word
  WGPU_CUDA(cudaMemcpyAsync(g->h_flags, g->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaStreamSynchronize(s));
  if (*g->h_flags != 0) {
    *g->h_flags = 0;
    WGPU_CUDA(cudaMemsetAsync(g->d_flags, 0, sizeof(unsigned), s));
    WGPU_CUDA(cudaStreamSynchronize(s));
    throw Error(WGPU_ERR_TIMEOUT, "a bounded device wait expired (bucket sort look-back)");
  }
  g->bound = std::move(b);
}

void invert_bound(wgpu_gridder *g, const float *vis, bool device) {
  if (!g->bound) throw Error(WGPU_ERR_STATE, "no bound visibility set");
  if (g->mode != wgpu_gridder::Mode::kInversion)
    throw Error(WGPU_ERR_STATE, "bound inversion before InitializeInversion");
  BoundState &b = *g->bound;
  cudaStream_t s = g->stream;
  g->timer.begin(s);
  g->timer.mark("bound_invert");
  if (device)
    WGPU_CUDA(cudaMemcpyAsync(b.vis_in, vis, sizeof(float2) * b.n_rows * b.n_chan,
                              cudaMemcpyDeviceToDevice, s));
  else
    copy_to_device(g, b.vis_in, vis, sizeof(float2) * b.n_rows * b.n_chan);
  WGPU_CUDA(cudaGraphLaunch(b.xinv, s));
  count_launch((int)b.inv_kernels);
  end_call(g);
  g->last_plan = b.plan;
}

void predict_bound(wgpu_gridder *g, float *vis, bool device) {
  if (!g->bound) throw Error(WGPU_ERR_STATE, "no bound visibility set");
  if (g->mode != wgpu_gridder::Mode::kPrediction)
    throw Error(WGPU_ERR_STATE, "bound prediction before InitializePrediction");
  BoundState &b = *g->bound;
  cudaStream_t s = g->stream;
  g->timer.begin(s);
  g->timer.mark("bound_predict");
  WGPU_CUDA(cudaGraphLaunch(b.xpred, s));
  count_launch((int)b.pred_kernels);
  if (device)
    WGPU_CUDA(cudaMemcpyAsync(vis, b.vis_out, sizeof(float2) * b.n_rows * b.n_chan,
                              cudaMemcpyDeviceToDevice, s));
  else
    copy_to_host(g, vis, b.vis_out, sizeof(float2) * b.n_rows * b.n_chan);
  end_call(g);
  g->last_plan = b.plan;
}

template <typename T>
T *upload(wgpu_gridder *g, int slot, const T *h, size_t n) {
  T *d = (T *)g->arena.get(slot, sizeof(T) * (n ? n : 1));
  copy_to_device(g, d, h, sizeof(T) * n);
  return d;
}

}  // namespace
}  // namespace wgpu

using namespace wgpu;

extern "C" {

const char *wgpu_last_error(void) { return g_last_error.c_str(); }

const char *wgpu_version(void) { return "wgpu 0.1 (sm_103a)"; }

size_t wgpu_gain_mode_n_visibilities(int mode) {
  switch (mode) {
    case WGPU_GAIN_XX:
    case WGPU_GAIN_YY:
    case WGPU_GAIN_TRACE:
      return 1;
    case WGPU_GAIN_2VIS_DIAGONAL:
      return 2;
    case WGPU_GAIN_FULL:
      return 4;
    default:
      return 0;
  }
}

int wgpu_select_gain_mode(int polarization, size_t n_visibility_polarizations, int *mode) {
  if (!mode) return fail(WGPU_ERR_INVALID, "null mode");
  if (polarization < WGPU_POL_STOKES_I || polarization > WGPU_POL_DIAGONAL_INSTRUMENTAL)
    return fail(WGPU_ERR_INVALID, "unknown polarization");
  const bool stokes = polarization <= WGPU_POL_STOKES_V;
  const bool xx_or_yy = polarization == WGPU_POL_XX || polarization == WGPU_POL_YY;
  switch (n_visibility_polarizations) {
    case 1:
      // every polarisation other than XX and YY (Stokes I, RR, other Stokes)
      // is corrected with the trace
      *mode = polarization == WGPU_POL_XX   ? WGPU_GAIN_XX
              : polarization == WGPU_POL_YY ? WGPU_GAIN_YY
                                            : WGPU_GAIN_TRACE;
      return WGPU_OK;
    case 2:
      if (polarization == WGPU_POL_STOKES_I || polarization == WGPU_POL_DIAGONAL_INSTRUMENTAL ||
          xx_or_yy) {
        *mode = WGPU_GAIN_2VIS_DIAGONAL;
        return WGPU_OK;
      }
      break;
    case 4:
      if (polarization == WGPU_POL_FULL_STOKES || polarization == WGPU_POL_INSTRUMENTAL ||
          stokes || xx_or_yy) {
        *mode = WGPU_GAIN_FULL;
        return WGPU_OK;
      }
      break;
  }
  return fail(WGPU_ERR_INVALID, "invalid combination of polarization (" +
                                    std::to_string(polarization) +
                                    ") and n_visibility_polarizations (" +
                                    std::to_string(n_visibility_polarizations) + ")");
}

int wgpu_plan_make(const wgpu_plan_request_t *request, wgpu_plan_t *plan) {
  if (!request || !plan) return fail(WGPU_ERR_INVALID, "null argument");
  return guarded([&] { *plan = make_plan(*request); });
}

int wgpu_plan_candidates(const wgpu_plan_request_t *request, wgpu_plan_t *plans, int max_plans,
                         int *n_plans) {
  if (!request || !n_plans || max_plans < 0 || (max_plans > 0 && !plans))
    return fail(WGPU_ERR_INVALID, "null argument or negative count");
  *n_plans = 0;
  return guarded([&] {
    const std::vector<wgpu_plan_t> c = plan_candidates(*request, (size_t)max_plans);
    const int n = (int)std::min<size_t>(c.size(), (size_t)max_plans);
    for (int i = 0; i < n; ++i) plans[i] = c[i];
    *n_plans = n;
  });
}

int wgpu_gridder_create(size_t width, size_t height, size_t width_t,
                        size_t height_t, double pixel_size_x,
                        double pixel_size_y, double l_shift, double m_shift,
                        size_t nthreads, double epsilon, size_t verbosity,
                        int tuning, int precision_bytes,
                        wgpu_gridder_t **gridder) {
  if (!gridder) return fail(WGPU_ERR_INVALID, "null gridder pointer");
  *gridder = nullptr;
  if (verbosity > 2) return fail(WGPU_ERR_INVALID, "verbosity must be 0, 1, or 2");
  if (precision_bytes != 4 && precision_bytes != 8)
    return fail(WGPU_ERR_INVALID, "precision_bytes must be 4 or 8");
  if (width_t > width || height_t > height || width_t == 0 || height_t == 0)
    return fail(WGPU_ERR_INVALID, "trimmed size must be non-zero and fit the image");
  if ((width_t & 1) || (height_t & 1))
    return fail(WGPU_ERR_INVALID, "trimmed image dimensions must be even");
  if (!(pixel_size_x > 0) || !(pixel_size_y > 0) || !(epsilon > 0))
    return fail(WGPU_ERR_INVALID, "pixel sizes and epsilon must be positive");
  return guarded([&] {
    int n_dev = 0;
    cudaError_t e = cudaGetDeviceCount(&n_dev);
    if (e != cudaSuccess || n_dev == 0) {
      cudaGetLastError();
      throw Error(WGPU_ERR_CUDA, std::string("no usable CUDA device: ") +
                                     (e != cudaSuccess ? cudaGetErrorString(e) : "count is 0"));
    }
    auto *g = new wgpu_gridder();
    g->width = width;
    g->height = height;
    g->width_t = width_t;
    g->height_t = height_t;
    g->dl = pixel_size_x;
    g->dm = pixel_size_y;
    g->l_shift = l_shift;
    g->m_shift = m_shift;
    g->nthreads = nthreads;
    g->epsilon = epsilon;
    g->verbosity = verbosity;
    g->tuning = tuning != 0;
    g->prec = precision_bytes;
    std::memset(&g->last_plan, 0, sizeof(g->last_plan));
    try {
      WGPU_CUDA(cudaGetDevice(&g->device));
      WGPU_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
      WGPU_CUDA(cudaMalloc(&g->d_flags, sizeof(unsigned)));
      WGPU_CUDA(cudaMemset(g->d_flags, 0, sizeof(unsigned)));
      WGPU_CUDA(cudaMallocHost(&g->h_flags, sizeof(unsigned)));
      *g->h_flags = 0;
      g->fft = fft_tables_create();
    } catch (...) {
      if (g->d_flags) cudaFree(g->d_flags);
      if (g->h_flags) cudaFreeHost(g->h_flags);
      if (g->stream) cudaStreamDestroy(g->stream);
      delete g;
      throw;
    }
    *gridder = g;
  });
}

void wgpu_gridder_destroy(wgpu_gridder_t *g) {
  if (!g) return;
  if (g->stream) cudaStreamSynchronize(g->stream);
  g->bound.reset();
  g->arena.release();
  if (g->d_img) cudaFree(g->d_img);
  if (g->d_flags) cudaFree(g->d_flags);
  if (g->h_flags) cudaFreeHost(g->h_flags);
  for (int k = 0; k < 2; ++k) {
    if (g->stage_buf[k]) cudaFreeHost(g->stage_buf[k]);
    if (g->stage_ev[k]) cudaEventDestroy(g->stage_ev[k]);
  }
  fft_tables_destroy(g->fft);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

// gridder_simple_implementation.h:53-61
size_t wgpu_gridder_constant_memory(const wgpu_gridder_t *g) {
  if (!g) return 0;
  const double sigma_max = 2.0;
  size_t c = (size_t)(sigma_max * sigma_max * g->width_t * g->height_t * 8.0);
  c += g->width_t * g->height_t * (size_t)g->prec;
  return c;
}

// gridder_simple_implementation.h:63-68
size_t wgpu_gridder_per_visibility_memory(const wgpu_gridder_t *) { return 8; }

int wgpu_gridder_initialize_inversion(wgpu_gridder_t *g) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  return guarded([&] {
    ensure_image(g);
    WGPU_CUDA(cudaMemsetAsync(g->d_img, 0, image_bytes(g), g->stream));
    g->mode = wgpu_gridder::Mode::kInversion;
  });
}

int wgpu_gridder_add_inversion_data_device(wgpu_gridder_t *g, size_t n_rows,
                                           size_t n_chan, const double *d_uvw,
                                           const double *d_freq,
                                           const float *d_vis) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  if ((n_rows && n_chan) && (!d_uvw || !d_freq || !d_vis))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] { invert_device(g, n_rows, n_chan, d_uvw, d_freq, d_vis); });
}

int wgpu_gridder_add_inversion_data(wgpu_gridder_t *g, size_t n_rows,
                                    size_t n_chan, const double *uvw,
                                    const double *freq, const float *vis) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  if ((n_rows && n_chan) && (!uvw || !freq || !vis))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] {
    if (g->mode != wgpu_gridder::Mode::kInversion)
      throw Error(WGPU_ERR_STATE, "AddInversionData before InitializeInversion");
    const double *du = upload(g, kSlotUvw, uvw, 3 * n_rows);
    const double *df = upload(g, kSlotFreq, freq, n_chan);
    const float *dv = upload(g, kSlotVis, vis, 2 * n_rows * n_chan);
    invert_device(g, n_rows, n_chan, du, df, dv);
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
  });
}

int wgpu_gridder_add_inversion_rows(wgpu_gridder_t *g, const wgpu_imageweights_t *iw,
                                    const wgpu_row_weighting_t *rw, size_t n_pol,
                                    size_t n_rows, size_t n_chan, const double *uvw,
                                    const double *freq, const float *vis,
                                    const float *weights, const float *model,
                                    const uint8_t *selected, wgpu_weight_sums_t *sums) {
  if (!g || !iw || !rw) return fail(WGPU_ERR_INVALID, "null argument");
  if (rw->psf_mode < WGPU_PSF_NONE || rw->psf_mode > WGPU_PSF_DIRECTION_DEPENDENT ||
      rw->visibility_weighting < WGPU_VISW_NORMAL || rw->visibility_weighting > WGPU_VISW_UNIT ||
      rw->polarization < 0 || rw->polarization > 7)
    return fail(WGPU_ERR_INVALID, "invalid row weighting");
  if (n_pol != 1 && n_pol != 2 && n_pol != 4)
    return fail(WGPU_ERR_INVALID, "n_pol must be 1, 2 or 4");
  if (n_rows && n_chan &&
      (!uvw || !freq || !weights || (rw->psf_mode == WGPU_PSF_NONE && !vis) ||
       (rw->subtract_model && !model)))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] {
    if (g->mode != wgpu_gridder::Mode::kInversion)
      throw Error(WGPU_ERR_STATE, "AddInversionData before InitializeInversion");
    if (n_rows == 0 || n_chan == 0) return;
    const size_t n = n_rows * n_chan, nc = n * n_pol;
    const double *du = upload(g, kSlotUvw, uvw, 3 * n_rows);
    const double *df = upload(g, kSlotFreq, freq, n_chan);
    const float *dw = upload(g, kSlotRowWeights, weights, nc);
    const float2 *dv =
        rw->psf_mode == WGPU_PSF_NONE ? (const float2 *)upload(g, kSlotGainVis, vis, 2 * nc)
                                      : nullptr;
    const float2 *dm =
        rw->subtract_model ? (const float2 *)upload(g, kSlotRowModel, model, 2 * nc) : nullptr;
    const uint8_t *ds = selected ? upload(g, kSlotRowSel, selected, n) : nullptr;
    float2 *dc = (float2 *)g->arena.get(kSlotVis, sizeof(float2) * n);
    auto *dsum = (WeightSumsDev *)g->arena.get(kSlotRowSums, sizeof(WeightSumsDev));
    void *work = g->arena.get(kSlotRowWork, pass_work_bytes((int64_t)n_rows, (int64_t)n_chan));
    const WeightGridView view = imageweights_view(iw);
    WGPU_CUDA(cudaMemsetAsync(dsum, 0, sizeof(WeightSumsDev), g->stream));
    launch_prepare_rows(view, row_weighting(*rw), (int)n_pol, (int64_t)n_rows, (int64_t)n_chan,
                        du, df, dv, dw, dm, ds, dc, nullptr, nullptr, dsum, work, g->stream);
    WeightSumsDev hs;
    WGPU_CUDA(cudaMemcpyAsync(&hs, dsum, sizeof(hs), cudaMemcpyDeviceToHost, g->stream));
    invert_device(g, n_rows, n_chan, du, df, (const float *)dc);
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
    add_weight_sums(hs, sums);
  });
}

int wgpu_gridder_add_inversion_rows_corrected(
    wgpu_gridder_t *g, const wgpu_imageweights_t *iw, const wgpu_row_weighting_t *rw, int mode,
    size_t n_pol, size_t n_rows, size_t n_chan, const double *uvw, const double *freq,
    const float *vis, const float *weights, const float *model, const uint8_t *selected,
    const uint64_t *antenna_pairs, const uint64_t *time_offsets, const float *solutions,
    size_t nparms, size_t n_times, size_t n_ant, wgpu_weight_sums_t *sums,
    double *correction_sum) {
  if (!g || !iw || !rw) return fail(WGPU_ERR_INVALID, "null argument");
  if (rw->psf_mode < WGPU_PSF_NONE || rw->psf_mode > WGPU_PSF_DIRECTION_DEPENDENT ||
      rw->visibility_weighting < WGPU_VISW_NORMAL || rw->visibility_weighting > WGPU_VISW_UNIT ||
      rw->polarization < 0 || rw->polarization > 7)
    return fail(WGPU_ERR_INVALID, "invalid row weighting");
  if (mode < WGPU_GAIN_XX || mode > WGPU_GAIN_FULL)
    return fail(WGPU_ERR_INVALID, "invalid gain mode");
  const size_t want = mode == WGPU_GAIN_FULL ? 4 : mode == WGPU_GAIN_2VIS_DIAGONAL ? 2 : 1;
  if (n_pol != want) return fail(WGPU_ERR_INVALID, "gain mode and n_polarizations do not match");
  if (nparms != 2 && nparms != 4) return fail(WGPU_ERR_INVALID, "nparms must be 2 or 4");
  if (n_rows && n_chan &&
      (!uvw || !freq || !weights || (rw->psf_mode == WGPU_PSF_NONE && !vis) ||
       (rw->subtract_model && !model) || !antenna_pairs || !time_offsets || !solutions))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] {
    if (g->mode != wgpu_gridder::Mode::kInversion)
      throw Error(WGPU_ERR_STATE, "AddInversionData before InitializeInversion");
    if (n_rows == 0 || n_chan == 0) return;
    const size_t n = n_rows * n_chan, nc = n * n_pol;
    const double *du = upload(g, kSlotUvw, uvw, 3 * n_rows);
    const double *df = upload(g, kSlotFreq, freq, n_chan);
    const float *dw = upload(g, kSlotRowWeights, weights, nc);
    const float2 *dv =
        rw->psf_mode == WGPU_PSF_NONE ? (const float2 *)upload(g, kSlotGainVis, vis, 2 * nc)
                                      : nullptr;
    const float2 *dm =
        rw->subtract_model ? (const float2 *)upload(g, kSlotRowModel, model, 2 * nc) : nullptr;
    const uint8_t *ds = selected ? upload(g, kSlotRowSel, selected, n) : nullptr;
    GainTable gt;
    gt.ant = upload(g, kSlotAnt, antenna_pairs, 2 * n_rows);
    gt.tof = upload(g, kSlotTimes, time_offsets, n_rows);
    gt.sol = (const float2 *)upload(g, kSlotSol, solutions, 2 * n_times * n_chan * n_ant * nparms);
    gt.nparms = (int)nparms;
    gt.mode = mode;
    gt.n_times = (int64_t)n_times;
    gt.n_ant = (int64_t)n_ant;
    gt.err = (int *)g->arena.get(kSlotOutVis, sizeof(int) * 4);
    gt.sum_matrix = correction_sum != nullptr && mode != WGPU_GAIN_TRACE;
    float2 *dc = (float2 *)g->arena.get(kSlotVis, sizeof(float2) * n);
    auto *dsum = (WeightSumsDev *)g->arena.get(kSlotRowSums, sizeof(WeightSumsDev));
    void *work = g->arena.get(kSlotRowWork, pass_work_bytes((int64_t)n_rows, (int64_t)n_chan));
    const WeightGridView view = imageweights_view(iw);
    WGPU_CUDA(cudaMemsetAsync(dsum, 0, sizeof(WeightSumsDev), g->stream));
    WGPU_CUDA(cudaMemsetAsync(gt.err, 0, sizeof(int), g->stream));
    launch_prepare_rows(view, row_weighting(*rw), (int)n_pol, (int64_t)n_rows, (int64_t)n_chan,
                        du, df, dv, dw, dm, ds, dc, nullptr, nullptr, dsum, work, g->stream, &gt);
    WeightSumsDev hs;
    int herr = 0;
    WGPU_CUDA(cudaMemcpyAsync(&hs, dsum, sizeof(hs), cudaMemcpyDeviceToHost, g->stream));
    WGPU_CUDA(cudaMemcpyAsync(&herr, gt.err, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
    if (herr) throw Error(WGPU_ERR_INVALID, "antenna index or time offset outside the solution table");
    invert_device(g, n_rows, n_chan, du, df, (const float *)dc);
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
    add_weight_sums(hs, sums);
    if (correction_sum) {
      if (mode == WGPU_GAIN_TRACE) {
        *correction_sum += hs.correction;
      } else {
        // the Hermitian matrix, row-major, (re, im) per element
        static const int kRow[6] = {0, 0, 0, 1, 1, 2}, kCol[6] = {1, 2, 3, 2, 3, 3};
        for (int d = 0; d < 4; ++d) correction_sum[2 * (d * 4 + d)] += hs.matrix[d];
        for (int e = 0; e < 6; ++e) {
          const double re = hs.matrix[4 + 2 * e], im = hs.matrix[5 + 2 * e];
          const int r = kRow[e], c = kCol[e];
          correction_sum[2 * (r * 4 + c)] += re;
          correction_sum[2 * (r * 4 + c) + 1] += im;
          correction_sum[2 * (c * 4 + r)] += re;
          correction_sum[2 * (c * 4 + r) + 1] -= im;
        }
      }
    }
  });
}

int wgpu_gridder_add_inversion_data_corrected(
    wgpu_gridder_t *g, int mode, size_t n_pol, size_t n_rows, const double *uvw,
    const double *freq, size_t n_chan, const uint64_t *antenna_pairs,
    const float *vis, const uint64_t *time_offsets, const float *solutions,
    size_t nparms, size_t n_times, size_t n_ant, int polarization) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  if (mode < WGPU_GAIN_XX || mode > WGPU_GAIN_FULL)
    return fail(WGPU_ERR_INVALID, "invalid gain mode");
  if (n_pol != 1 && n_pol != 2 && n_pol != 4)
    return fail(WGPU_ERR_INVALID, "n_polarizations must be 1, 2 or 4");
  const size_t want = mode == WGPU_GAIN_FULL ? 4 : mode == WGPU_GAIN_2VIS_DIAGONAL ? 2 : 1;
  if (n_pol != want)
    return fail(WGPU_ERR_INVALID, "gain mode and n_polarizations do not match");
  if (nparms != 2 && nparms != 4) return fail(WGPU_ERR_INVALID, "nparms must be 2 or 4");
  if (polarization < 0 || polarization > 7) return fail(WGPU_ERR_INVALID, "invalid polarization");
  if ((n_rows && n_chan) && (!uvw || !freq || !vis || !antenna_pairs || !time_offsets || !solutions))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] {
    if (g->mode != wgpu_gridder::Mode::kInversion)
      throw Error(WGPU_ERR_STATE, "AddInversionData before InitializeInversion");
    if (n_rows == 0 || n_chan == 0) return;
    const double *du = upload(g, kSlotUvw, uvw, 3 * n_rows);
    const double *df = upload(g, kSlotFreq, freq, n_chan);
    const float *dv = upload(g, kSlotGainVis, vis, 2 * n_rows * n_chan * n_pol);
    const uint64_t *da = upload(g, kSlotAnt, antenna_pairs, 2 * n_rows);
    const uint64_t *dt = upload(g, kSlotTimes, time_offsets, n_rows);
    const float *ds = upload(g, kSlotSol, solutions, 2 * n_times * n_chan * n_ant * nparms);
    float2 *dc = (float2 *)g->arena.get(kSlotVis, sizeof(float2) * n_rows * n_chan);
    int *err = (int *)g->arena.get(kSlotOutVis, sizeof(int) * 4);
    WGPU_CUDA(cudaMemsetAsync(err, 0, sizeof(int), g->stream));
    launch_apply_gains(mode, (int)n_pol, (int64_t)n_rows, (int64_t)n_chan,
                       (const float2 *)dv, da, dt, (const float2 *)ds, (int)nparms,
                       (int64_t)n_times, (int64_t)n_ant, polarization, dc, err, g->stream);
    int herr = 0;
    WGPU_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
    if (herr) throw Error(WGPU_ERR_INVALID, "antenna index or time offset outside the solution table");
    invert_device(g, n_rows, n_chan, du, df, (const float *)dc);
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
  });
}

int wgpu_gridder_predict_visibilities_corrected(
    wgpu_gridder_t *g, int mode, size_t n_pol, size_t n_rows, const double *uvw,
    const double *freq, size_t n_chan, const uint64_t *antenna_pairs,
    const uint64_t *time_offsets, const float *solutions, size_t nparms, size_t n_times,
    size_t n_ant, int polarization, float *vis) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  if (mode < WGPU_GAIN_XX || mode > WGPU_GAIN_FULL)
    return fail(WGPU_ERR_INVALID, "invalid gain mode");
  if (n_pol != 1 && n_pol != 2 && n_pol != 4)
    return fail(WGPU_ERR_INVALID, "n_polarizations must be 1, 2 or 4");
  const size_t want = mode == WGPU_GAIN_FULL ? 4 : mode == WGPU_GAIN_2VIS_DIAGONAL ? 2 : 1;
  if (n_pol != want)
    return fail(WGPU_ERR_INVALID, "gain mode and n_polarizations do not match");
  if (nparms != 2 && nparms != 4) return fail(WGPU_ERR_INVALID, "nparms must be 2 or 4");
  if (polarization < 0 || polarization > 7) return fail(WGPU_ERR_INVALID, "invalid polarization");
  if ((n_rows && n_chan) && (!uvw || !freq || !vis || !antenna_pairs || !time_offsets || !solutions))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] {
    if (g->mode != wgpu_gridder::Mode::kPrediction)
      throw Error(WGPU_ERR_STATE, "PredictVisibilities before InitializePrediction");
    if (n_rows == 0 || n_chan == 0) return;
    const double *du = upload(g, kSlotUvw, uvw, 3 * n_rows);
    const double *df = upload(g, kSlotFreq, freq, n_chan);
    const uint64_t *da = upload(g, kSlotAnt, antenna_pairs, 2 * n_rows);
    const uint64_t *dt = upload(g, kSlotTimes, time_offsets, n_rows);
    const float *ds = upload(g, kSlotSol, solutions, 2 * n_times * n_chan * n_ant * nparms);
    float2 *dp = (float2 *)g->arena.get(kSlotVis, sizeof(float2) * n_rows * n_chan);
    float2 *dout = (float2 *)g->arena.get(kSlotGainVis, sizeof(float2) * n_rows * n_chan * n_pol);
    int *err = (int *)g->arena.get(kSlotOutVis, sizeof(int) * 4);
    predict_device(g, n_rows, n_chan, du, df, nullptr, (float *)dp);
    WGPU_CUDA(cudaMemsetAsync(err, 0, sizeof(int), g->stream));
    launch_forward_gains(mode, (int)n_pol, (int64_t)n_rows, (int64_t)n_chan, dp, da, dt,
                         (const float2 *)ds, (int)nparms, (int64_t)n_times, (int64_t)n_ant,
                         polarization, dout, err, g->stream);
    int herr = 0;
    WGPU_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    copy_to_host(g, vis, dout, sizeof(float2) * n_rows * n_chan * n_pol);
    if (herr) throw Error(WGPU_ERR_INVALID, "antenna index or time offset outside the solution table");
  });
}

int wgpu_gridder_finalize_image(wgpu_gridder_t *g, double factor) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  return guarded([&] {
    if (!g->d_img) throw Error(WGPU_ERR_STATE, "FinalizeImage without an image");
    launch_scale_image(g->d_img, g->prec, (int64_t)(g->width_t * g->height_t), factor, g->stream);
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
  });
}

int wgpu_gridder_real_image(wgpu_gridder_t *g, float *image) {
  if (!g || !image) return fail(WGPU_ERR_INVALID, "null argument");
  return guarded([&] {
    if (!g->d_img) throw Error(WGPU_ERR_STATE, "RealImage without an image");
    // trimmed image -> full float image with NaN borders on the device, then
    // one copy to the caller
    const int64_t n = (int64_t)(g->width * g->height);
    float *d_out = (float *)g->arena.get(kSlotImgIO, sizeof(float) * (size_t)n);
    image_out_kernel<<<(unsigned)((n + 255) / 256), 256, 0, g->stream>>>(
        g->d_img, g->prec, (int64_t)g->width_t, (int64_t)g->height_t, (int64_t)g->width,
        (int64_t)g->height, d_out);
    check_launch("image_out_kernel");
    copy_to_host(g, image, d_out, sizeof(float) * (size_t)n);
  });
}

int wgpu_gridder_initialize_prediction(wgpu_gridder_t *g, const float *image) {
  if (!g || !image) return fail(WGPU_ERR_INVALID, "null argument");
  return guarded([&] {
    ensure_image(g);
    // the caller's float image to the device, then its trimmed region into
    // the gridder's image (float or double)
    const int64_t n = (int64_t)(g->width * g->height);
    float *d_in = (float *)g->arena.get(kSlotImgIO, sizeof(float) * (size_t)n);
    copy_to_device(g, d_in, image, sizeof(float) * (size_t)n);
    const int64_t nt = (int64_t)(g->width_t * g->height_t);
    image_in_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, g->stream>>>(
        d_in, g->prec, (int64_t)g->width_t, (int64_t)g->height_t, (int64_t)g->width,
        (int64_t)g->height, g->d_img);
    check_launch("image_in_kernel");
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
    g->mode = wgpu_gridder::Mode::kPrediction;
  });
}

int wgpu_gridder_finish_inversion(wgpu_gridder_t *g, size_t image_width, size_t image_height,
                                  size_t trim_width, size_t trim_height, float *image) {
  if (!g || !image) return fail(WGPU_ERR_INVALID, "null argument");
  if (!image_width || !image_height || trim_width > image_width || trim_height > image_height ||
      !trim_width || !trim_height || image_width > 65536 || image_height > 65536)
    return fail(WGPU_ERR_INVALID, "invalid image or trim size");
  return guarded([&] {
    if (!g->d_img) throw Error(WGPU_ERR_STATE, "FinishInversion without an image");
    cudaStream_t s = g->stream;
    // RealImage at the inversion size (NaN outside the gridder's trimmed
    // region), resampled to the image size, trimmed (wgriddingmsgridder.cpp:
    // 285-309)
    const int64_t w = (int64_t)g->width, h = (int64_t)g->height;
    float *d_full = (float *)g->arena.get(kSlotImgIO, sizeof(float) * (size_t)(w * h));
    image_out_kernel<<<(unsigned)((w * h + 255) / 256), 256, 0, s>>>(
        g->d_img, g->prec, (int64_t)g->width_t, (int64_t)g->height_t, w, h, d_full);
    check_launch("image_out_kernel");
    const float *src = d_full;
    int64_t sw = w, sh = h;
    if ((int64_t)image_width != w || (int64_t)image_height != h) {
      float *d_rs = (float *)g->arena.get(kSlotResampleOut,
                                          sizeof(float) * image_width * image_height);
      void *work = g->arena.get(kSlotResampleWork,
                                resample_work_bytes(w, h, image_width, image_height));
      resample_device(d_full, w, h, d_rs, (int64_t)image_width, (int64_t)image_height, work, s);
      src = d_rs;
      sw = (int64_t)image_width;
      sh = (int64_t)image_height;
    }
    if ((int64_t)trim_width != sw || (int64_t)trim_height != sh) {
      float *d_t = (float *)g->arena.get(kSlotResampleTrim,
                                         sizeof(float) * trim_width * trim_height);
      launch_trim(src, sw, sh, d_t, (int64_t)trim_width, (int64_t)trim_height, s);
      src = d_t;
    }
    copy_to_host(g, image, src, sizeof(float) * trim_width * trim_height);
  });
}

int wgpu_gridder_start_predict(wgpu_gridder_t *g, size_t trim_width, size_t trim_height,
                               size_t image_width, size_t image_height, const float *model) {
  if (!g || !model) return fail(WGPU_ERR_INVALID, "null argument");
  if (!image_width || !image_height || trim_width > image_width || trim_height > image_height ||
      !trim_width || !trim_height || image_width > 65536 || image_height > 65536)
    return fail(WGPU_ERR_INVALID, "invalid image or trim size");
  return guarded([&] {
    ensure_image(g);
    cudaStream_t s = g->stream;
    // untrim to the image size, resample to the inversion size, then the
    // gridder's InitializePrediction (wgriddingmsgridder.cpp:311-340)
    const int64_t w = (int64_t)g->width, h = (int64_t)g->height;
    float *d_m = (float *)g->arena.get(kSlotResampleTrim, sizeof(float) * trim_width * trim_height);
    copy_to_device(g, d_m, model, sizeof(float) * trim_width * trim_height);
    const float *src = d_m;
    int64_t sw = (int64_t)trim_width, sh = (int64_t)trim_height;
    if (trim_width != image_width || trim_height != image_height) {
      float *d_u = (float *)g->arena.get(kSlotResampleOut,
                                         sizeof(float) * image_width * image_height);
      launch_untrim(d_m, sw, sh, d_u, (int64_t)image_width, (int64_t)image_height, s);
      src = d_u;
      sw = (int64_t)image_width;
      sh = (int64_t)image_height;
    }
    if (sw != w || sh != h) {
      float *d_full = (float *)g->arena.get(kSlotImgIO, sizeof(float) * (size_t)(w * h));
      void *work = g->arena.get(kSlotResampleWork, resample_work_bytes(sw, sh, w, h));
      resample_device(src, sw, sh, d_full, w, h, work, s);
      src = d_full;
    }
    const int64_t nt = (int64_t)(g->width_t * g->height_t);
    image_in_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(
        src, g->prec, (int64_t)g->width_t, (int64_t)g->height_t, w, h, g->d_img);
    check_launch("image_in_kernel");
    WGPU_CUDA(cudaStreamSynchronize(s));
    g->mode = wgpu_gridder::Mode::kPrediction;
  });
}

int wgpu_gridder_predict_visibilities_device(wgpu_gridder_t *g, size_t n_rows,
                                             size_t n_chan, const double *d_uvw,
                                             const double *d_freq, float *d_vis) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  if ((n_rows && n_chan) && (!d_uvw || !d_freq || !d_vis))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] { predict_device(g, n_rows, n_chan, d_uvw, d_freq, nullptr, d_vis); });
}

int wgpu_gridder_predict_visibilities_masked_device(
    wgpu_gridder_t *g, size_t n_rows, size_t n_chan, const double *d_uvw,
    const double *d_freq, const uint8_t *d_mask, float *d_vis) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  if ((n_rows && n_chan) && (!d_uvw || !d_freq || !d_vis || !d_mask))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] { predict_device(g, n_rows, n_chan, d_uvw, d_freq, d_mask, d_vis); });
}

int wgpu_gridder_predict_visibilities_masked(wgpu_gridder_t *g, size_t n_rows,
                                             size_t n_chan, const double *uvw,
                                             const double *freq,
                                             const uint8_t *mask, float *vis) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  if ((n_rows && n_chan) && (!uvw || !freq || !vis || !mask))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] {
    if (g->mode != wgpu_gridder::Mode::kPrediction)
      throw Error(WGPU_ERR_STATE, "PredictVisibilities before InitializePrediction");
    if (n_rows == 0 || n_chan == 0) return;
    const double *du = upload(g, kSlotUvw, uvw, 3 * n_rows);
    const double *df = upload(g, kSlotFreq, freq, n_chan);
    const uint8_t *dm = upload(g, kSlotAnt, mask, n_rows * n_chan);
    float *dv = (float *)g->arena.get(kSlotVis, sizeof(float2) * n_rows * n_chan);
    predict_device(g, n_rows, n_chan, du, df, dm, dv);
    copy_to_host(g, vis, dv, sizeof(float2) * n_rows * n_chan);
  });
}

int wgpu_gridder_predict_visibilities(wgpu_gridder_t *g, size_t n_rows,
                                      size_t n_chan, const double *uvw,
                                      const double *freq, float *vis) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  if ((n_rows && n_chan) && (!uvw || !freq || !vis))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] {
    if (g->mode != wgpu_gridder::Mode::kPrediction)
      throw Error(WGPU_ERR_STATE, "PredictVisibilities before InitializePrediction");
    if (n_rows == 0 || n_chan == 0) return;
    const double *du = upload(g, kSlotUvw, uvw, 3 * n_rows);
    const double *df = upload(g, kSlotFreq, freq, n_chan);
    float *dv = (float *)g->arena.get(kSlotVis, sizeof(float2) * n_rows * n_chan);
    predict_device(g, n_rows, n_chan, du, df, nullptr, dv);
    copy_to_host(g, vis, dv, sizeof(float2) * n_rows * n_chan);
  });
}

int wgpu_gridder_last_plan(const wgpu_gridder_t *g, wgpu_plan_t *plan) {
  if (!g || !plan) return fail(WGPU_ERR_INVALID, "null argument");
  *plan = g->last_plan;
  return WGPU_OK;
}

int wgpu_gridder_pin_plan(wgpu_gridder_t *g, const wgpu_plan_t *plan) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  if (!plan) {
    g->pinned = false;
    return WGPU_OK;
  }
  if (plan->support < 2 || plan->support > kMaxSupport || plan->n_planes < 1 ||
      (plan->tile != 16 && plan->tile != 32) || plan->nu % plan->tile || plan->nv % plan->tile ||
      plan->nu < 2 * plan->tile || plan->nv < 2 * plan->tile || plan->support > plan->tile ||
      plan->plane_batch < 1 || plan->fft_n1 * plan->fft_n2 != plan->nv ||
      (plan->n_planes > 1 && plan->n_planes < plan->support))
    return fail(WGPU_ERR_INVALID, "pinned plan is not self-consistent");
  g->pinned_plan = *plan;
  g->pinned = true;
  return WGPU_OK;
}

int wgpu_gridder_last_tuning(const wgpu_gridder_t *g, wgpu_tuning_trial_t *trials,
                             int max_trials, int *n_trials) {
  if (!g || !n_trials || max_trials < 0 || (max_trials > 0 && !trials))
    return fail(WGPU_ERR_INVALID, "null argument or negative count");
  const int n = (int)std::min<size_t>(g->last_trials.size(), (size_t)max_trials);
  for (int i = 0; i < n; ++i) trials[i] = g->last_trials[i];
  *n_trials = n;
  return WGPU_OK;
}

void wgpu_tuning_cache_clear(void) { wgpu::tuning_cache_clear(); }

int wgpu_gridder_last_timings(const wgpu_gridder_t *g, double *ms, int *counts,
                              int max_entries, char *names, size_t names_len,
                              int *n_entries) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  std::string all;
  int n = 0;
  for (const auto &st : g->last_timings) {
    if (n < max_entries && ms) ms[n] = st.ms;
    if (n < max_entries && counts) counts[n] = st.count;
    if (n) all += ";";
    all += st.name;
    ++n;
  }
  if (n_entries) *n_entries = n;
  if (names && names_len) {
    std::strncpy(names, all.c_str(), names_len - 1);
    names[names_len - 1] = '\0';
  }
  return WGPU_OK;
}

void *wgpu_gridder_stream(wgpu_gridder_t *g) { return g ? (void *)g->stream : nullptr; }

uint64_t wgpu_kernel_launch_count(void) { return launch_count(); }

int wgpu_selftest_bounded_wait(double timeout_ms) {
  if (!(timeout_ms > 0) || timeout_ms > 10000)
    return fail(WGPU_ERR_INVALID, "timeout must be in (0, 10000] ms");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(WGPU_ERR_CUDA, "no usable CUDA device");
  }
  int st = WGPU_OK;
  const int g = guarded([&] { st = bounded_wait_selftest(timeout_ms); });
  if (g != WGPU_OK) return g;
  if (st == WGPU_ERR_TIMEOUT) return fail(st, "bounded device wait expired (self-test)");
  return st;
}

int wgpu_gridder_set_plane_budget(wgpu_gridder_t *g, double bytes) {
  return guarded([&] {
    if (!g) throw Error(WGPU_ERR_INVALID, "null gridder");
    if (!(bytes >= 0)) throw Error(WGPU_ERR_INVALID, "negative plane budget");
    g->plane_budget = bytes;
  });
}

int wgpu_gridder_bind(wgpu_gridder_t *g, size_t n_rows, size_t n_chan, const double *uvw,
                      const double *freq, const uint8_t *mask) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  if (!uvw || !freq) return fail(WGPU_ERR_INVALID, "null data pointer");
  return guarded([&] { bind_visibilities(g, n_rows, n_chan, uvw, freq, mask); });
}

int wgpu_gridder_unbind(wgpu_gridder_t *g) {
  if (!g) return fail(WGPU_ERR_INVALID, "null gridder");
  return guarded([&] {
    if (g->stream) WGPU_CUDA(cudaStreamSynchronize(g->stream));
    g->bound.reset();
  });
}

int wgpu_gridder_invert_bound(wgpu_gridder_t *g, const float *vis) {
  if (!g || !vis) return fail(WGPU_ERR_INVALID, "null argument");
  return guarded([&] {
    invert_bound(g, vis, false);
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
  });
}

int wgpu_gridder_invert_bound_device(wgpu_gridder_t *g, const float *d_vis) {
  if (!g || !d_vis) return fail(WGPU_ERR_INVALID, "null argument");
  return guarded([&] { invert_bound(g, d_vis, true); });
}

int wgpu_gridder_predict_bound(wgpu_gridder_t *g, float *vis) {
  if (!g || !vis) return fail(WGPU_ERR_INVALID, "null argument");
  return guarded([&] {
    predict_bound(g, vis, false);
    WGPU_CUDA(cudaStreamSynchronize(g->stream));
  });
}

int wgpu_gridder_predict_bound_device(wgpu_gridder_t *g, float *d_vis) {
  if (!g || !d_vis) return fail(WGPU_ERR_INVALID, "null argument");
  return guarded([&] { predict_bound(g, d_vis, true); });
}

static int bucket_debug_impl(const wgpu_plan_t *plan, size_t n_rows, size_t n_chan,
                             const double *uvw, const double *freq, const float *vis,
                             int skip_zero, uint32_t *perm, int32_t *iu, int32_t *iv,
                             int32_t *ip, float *fu, float *fv, float *fw, uint32_t *offsets,
                             int64_t *n_out, uint8_t *row_flags, uint32_t *row_start,
                             uint32_t *row_list) {
  if (!plan || !uvw || !freq) return fail(WGPU_ERR_INVALID, "null argument");
  if (skip_zero && !vis) return fail(WGPU_ERR_INVALID, "inversion bucketing needs vis");
  return guarded([&] {
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev == 0) {
      cudaGetLastError();
      throw Error(WGPU_ERR_CUDA, "no usable CUDA device");
    }
    DeviceArena arena;
    cudaStream_t s;
    WGPU_CUDA(cudaStreamCreate(&s));
    try {
      const DevPlan dp = to_dev_plan(*plan);
      double *du = (double *)arena.get(kSlotUvw, sizeof(double) * 3 * n_rows);
      double *df = (double *)arena.get(kSlotFreq, sizeof(double) * n_chan);
      float *dv = nullptr;
      WGPU_CUDA(cudaMemcpyAsync(du, uvw, sizeof(double) * 3 * n_rows, cudaMemcpyHostToDevice, s));
      WGPU_CUDA(cudaMemcpyAsync(df, freq, sizeof(double) * n_chan, cudaMemcpyHostToDevice, s));
      if (vis) {
        dv = (float *)arena.get(kSlotVis, sizeof(float2) * n_rows * n_chan);
        WGPU_CUDA(cudaMemcpyAsync(dv, vis, sizeof(float2) * n_rows * n_chan, cudaMemcpyHostToDevice, s));
      }
      const BucketResult b = bucket_visibilities(arena, dp, du, df, dv, nullptr, (int64_t)n_rows,
                                                 (int64_t)n_chan, skip_zero != 0, nullptr, s);
      std::vector<VisRecord> rec(b.n_out);
      if (b.n_out) {
        WGPU_CUDA(cudaMemcpyAsync(rec.data(), b.records, sizeof(VisRecord) * b.n_out, cudaMemcpyDeviceToHost, s));
        if (perm) WGPU_CUDA(cudaMemcpyAsync(perm, b.perm, sizeof(uint32_t) * b.n_out, cudaMemcpyDeviceToHost, s));
      }
      if (offsets)
        WGPU_CUDA(cudaMemcpyAsync(offsets, b.offsets, sizeof(uint32_t) * (b.n_keys + 1), cudaMemcpyDeviceToHost, s));
      WGPU_CUDA(cudaStreamSynchronize(s));
      for (int64_t k = 0; k < b.n_out; ++k) {
        if (iu) iu[k] = rec[k].iu;
        if (iv) iv[k] = rec[k].iv;
        if (ip) ip[k] = rec[k].ip;
        if (fu) fu[k] = rec[k].fu;
        if (fv) fv[k] = rec[k].fv;
        if (fw) fw[k] = rec[k].fw;
      }
      const RowOccupancy &o = b.rows;
      if (row_flags)
        WGPU_CUDA(cudaMemcpy(row_flags, o.flags(), o.cells(), cudaMemcpyDeviceToHost));
      std::vector<uint32_t> st((size_t)o.n_planes + 1, 0);
      if (o.n_planes > 0)
        WGPU_CUDA(cudaMemcpy(st.data(), o.start(), sizeof(uint32_t) * st.size(),
                             cudaMemcpyDeviceToHost));
      if (row_start) std::copy(st.begin(), st.end(), row_start);
      if (row_list && st.back() > 0)
        WGPU_CUDA(cudaMemcpy(row_list, o.list(), sizeof(uint32_t) * st.back(),
                             cudaMemcpyDeviceToHost));
      if (n_out) *n_out = b.n_out;
    } catch (...) {
      cudaStreamDestroy(s);
      throw;
    }
    cudaStreamDestroy(s);
  });
}


int wgpu_bucket_debug(const wgpu_plan_t *plan, size_t n_rows, size_t n_chan,
                      const double *uvw, const double *freq, const float *vis,
                      int skip_zero, uint32_t *perm, int32_t *iu, int32_t *iv,
                      int32_t *ip, float *fu, float *fv, float *fw,
                      uint32_t *offsets, int64_t *n_out) {
  if (!n_out) return fail(WGPU_ERR_INVALID, "null argument");
  return bucket_debug_impl(plan, n_rows, n_chan, uvw, freq, vis, skip_zero, perm, iu, iv, ip,
                           fu, fv, fw, offsets, n_out, nullptr, nullptr, nullptr);
}

int wgpu_bucket_debug_rows(const wgpu_plan_t *plan, size_t n_rows, size_t n_chan,
                           const double *uvw, const double *freq, const float *vis,
                           int skip_zero, uint8_t *row_flags, uint32_t *row_start,
                           uint32_t *row_list) {
  return bucket_debug_impl(plan, n_rows, n_chan, uvw, freq, vis, skip_zero, nullptr, nullptr,
                           nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                           row_flags, row_start, row_list);
}

}  // extern "C"

extern "C" {

size_t wgpu_bucket_noalloc_scratch_bytes(void) { return bucket_noalloc_scratch_bytes(); }

int wgpu_bucket_noalloc(const wgpu_plan_t *plan, size_t n_rows, size_t n_chan,
                        const double *d_uvw, const double *d_freq, const float *d_vis,
                        int skip_zero, void *d_records, uint32_t *d_perm, uint32_t *d_offsets,
                        void *stream, int64_t *n_out) {
  if (!plan || !n_out) return fail(WGPU_ERR_INVALID, "null argument");
  if ((n_rows && n_chan) && (!d_uvw || !d_freq || !d_records || !d_perm))
    return fail(WGPU_ERR_INVALID, "null data pointer");
  if (!d_offsets) return fail(WGPU_ERR_INVALID, "null offsets pointer");
  if (skip_zero && !d_vis && n_rows && n_chan)
    return fail(WGPU_ERR_INVALID, "inversion bucketing needs the visibilities");
  // the limits before any product of the sizes (which could wrap)
  if (n_chan > (size_t)WGPU_NOALLOC_MAX_CHANNELS)
    return fail(WGPU_ERR_INVALID, "allocation-free bucketing takes at most " +
                                      std::to_string(WGPU_NOALLOC_MAX_CHANNELS) + " channels");
  if (n_rows > (size_t)WGPU_NOALLOC_MAX_VISIBILITIES ||
      (n_chan != 0 && n_rows > (size_t)WGPU_NOALLOC_MAX_VISIBILITIES / n_chan))
    return fail(WGPU_ERR_INVALID, "allocation-free bucketing takes at most " +
                                      std::to_string(WGPU_NOALLOC_MAX_VISIBILITIES) +
                                      " visibilities");
  return guarded([&] {
    const DevPlan dp = to_dev_plan(*plan);
    *n_out = bucket_visibilities_noalloc(dp, d_uvw, d_freq, d_vis, (int64_t)n_rows,
                                         (int64_t)n_chan, skip_zero != 0, (VisRecord *)d_records,
                                         d_perm, d_offsets, (cudaStream_t)stream);
  });
}

}  // extern "C"
