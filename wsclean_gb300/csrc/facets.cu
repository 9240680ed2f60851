// Batched facets: many gridding jobs (facets of their own size and phase
// centre, times output-channel groups) on one visibility set.
//
// This is the GPU counterpart of WSClean's shared-read batch inversion
// (MSGridderManager::BatchInvert / ReadChunkForInvertImplementation,
// gridding/msgriddermanager.cpp:118-396), which runs one gridder per facet on
// the same chunk of rows, and of the per-facet l/m shifts of
// GriddingTaskFactory (scheduling/griddingtaskfactory.cpp:24-34).
//
// bind: the rows are uploaded once; each job is planned with a support width
// common to all jobs (chosen by summing the cost model over the jobs for every
// candidate width), bucketed into its own records, and given the work items of
// each of its plane batches.  The (job, plane batch) pairs are packed into
// waves that fit the plane-memory budget.  The whole inversion is captured in
// one CUDA graph: per job the visibilities are stamped into its records; per
// wave ONE persistent gridding launch works through the items of every pair in
// the wave, then each pair's FFT passes accumulate into its job's image (the
// pairs' FFT chains spread over four streams, joined before the next wave);
// per job the grid correction finishes the image.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "wgpu_internal.h"

namespace wgpu {
namespace {

constexpr int kFacetThreads = 256;

// records of a job from the visibilities of its channel range [c0, c0 + nch)
__global__ void restamp_channels_kernel(const VisRecord *__restrict__ geom,
                                        const uint32_t *__restrict__ perm,
                                        const float2 *__restrict__ vis, int64_t n, int nch,
                                        int n_chan, int c0, VisRecord *__restrict__ out) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const float4 a = __ldg(reinterpret_cast<const float4 *>(geom + s));
  const float4 b = __ldg(reinterpret_cast<const float4 *>(geom + s) + 1);
  const uint32_t e = __ldg(perm + s);
  const uint32_t row = e / (uint32_t)nch, ch = e - row * (uint32_t)nch;
  const float2 v = __ldg(vis + (size_t)row * n_chan + c0 + ch);
  // (a.x, a.y) is the sample's phase factor exp(-2 pi i theta)
  reinterpret_cast<float4 *>(out + s)[0] =
      make_float4(v.x * a.x - v.y * a.y, v.x * a.y + v.y * a.x, a.z, a.w);
  reinterpret_cast<float4 *>(out + s)[1] = b;
}

struct Job {
  wgpu_facet_t facet;
  int c0 = 0, nch = 0;
  double w_min = 0, w_max = 0;
  int64_t count = 0;
  wgpu_plan_t plan;
  DevPlan dp;
  int64_t n_out = 0;
  int64_t n_keys = 0;
  VisRecord *geom = nullptr, *work = nullptr;
  uint32_t *perm = nullptr, *offsets = nullptr;
  RowOccupancy rows_occ;  // plane rows the job's footprints touch
  float2 *acc = nullptr;
  double *nu_w = nullptr;
  ScreenTable scr;
  float *cx = nullptr, *cy = nullptr, *gl = nullptr, *wcorr = nullptr;
  float *img = nullptr;  // width * height, row-major
  std::vector<WorkItems> items;  // per plane batch
  int rstride = 0;
};

struct Slot {
  int job, batch, p0, nb;
  size_t planes_off, rows_off, spill_off;  // in float2 elements of the pool
};

}  // namespace
}  // namespace wgpu

using namespace wgpu;

namespace {
using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t).count();
}
}  // namespace

struct wgpu_facets {
  std::vector<wgpu_facet_t> facets;
  std::vector<size_t> groups;  // channel boundaries, n_groups + 1
  double epsilon = 1e-4;
  double plane_budget = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  static constexpr int kSide = 4;  // streams of the per-job FFT chains
  cudaStream_t side[kSide] = {};
  cudaEvent_t ev_grid = nullptr, ev_side[kSide] = {};
  FftTables *fft = nullptr;
  std::vector<Job> jobs;
  size_t n_rows = 0, n_chan = 0;
  double *d_uvw = nullptr, *d_freq = nullptr;
  float2 *d_vis = nullptr;
  // per-facet corrections: each facet's corrected, collapsed visibilities
  // (restamped by that facet's jobs), the shared uncorrected inputs
  bool per_facet = false;
  std::vector<float2 *> d_vis_facet;
  float *d_vis_raw = nullptr;
  size_t vis_raw_floats = 0;
  uint64_t *d_ant = nullptr, *d_tof = nullptr;
  float *d_sol = nullptr;
  size_t sol_floats = 0;
  int *d_err = nullptr;
  float *d_images = nullptr;
  size_t image_elems = 0;
  float2 *pool = nullptr;
  std::vector<std::vector<Slot>> waves;
  int support = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t graph_kernels = 0;
  unsigned *d_flags = nullptr, *h_flags = nullptr;
  bool bound = false;
  double last_ms = 0;
  // host time of the last bind's phases: upload, extents and planning;
  // bucketing and per-job tables; waves; graph capture and instantiation
  double bind_ms[4] = {};

  // Device memory of the bound state: regions bumped out of chunks that
  // outlive a bind, so that re-binding the batch (the next channel group, the
  // next chunk of rows) reuses them instead of allocating and freeing each
  // buffer.  Every region starts on a 512-byte boundary (the row transforms
  // read planes with 16-byte bulk copies and vector loads).
  struct Chunk {
    char *base;
    size_t size, used;
  };
  std::vector<Chunk> chunks;
  static constexpr size_t kChunkMin = 256ull << 20;
  DeviceArena scratch;  // bucketing scratch, kept across binds

  void *alloc(size_t bytes) {
    bytes = (std::max<size_t>(bytes, 16) + 511) & ~size_t(511);
    for (Chunk &c : chunks)
      if (c.size - c.used >= bytes) {
        void *p = c.base + c.used;
        c.used += bytes;
        return p;
      }
    size_t want = std::max(bytes, kChunkMin);
    char *p = nullptr;
    if (cudaMalloc(&p, want) != cudaSuccess) {
      cudaGetLastError();
      want = bytes;
      const cudaError_t e = cudaMalloc(&p, want);
      if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(WGPU_ERR_NOMEM, "device allocation of " + std::to_string(bytes) +
                                        " bytes failed: " + cudaGetErrorString(e));
      }
    }
    chunks.push_back(Chunk{p, want, bytes});
    return p;
  }
  // Ends the bound state.  Its memory stays for the next bind; when the last
  // bind needed more than one chunk, the chunks are merged into one of the
  // size it used (plus an eighth) so that a similar bind fits without growing.
  void release(bool keep_memory = true) {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    jobs.clear();
    waves.clear();
    bound = false;
    size_t used = 0;
    for (const Chunk &c : chunks) used += c.used;
    if (!keep_memory || chunks.size() > 1) {
      if (!chunks.empty() && stream) cudaStreamSynchronize(stream);
      for (const Chunk &c : chunks) cudaFree(c.base);
      chunks.clear();
      if (keep_memory && used > 0) {
        const size_t want = (used + used / 8 + 511) & ~size_t(511);
        char *p = nullptr;
        if (cudaMalloc(&p, want) == cudaSuccess)
          chunks.push_back(Chunk{p, want, 0});
        else
          cudaGetLastError();
      }
    }
    for (Chunk &c : chunks) c.used = 0;
    if (!keep_memory) scratch.release();
  }
  ~wgpu_facets() {
    if (stream) cudaStreamSynchronize(stream);
    release(false);
    if (d_flags) cudaFree(d_flags);
    if (h_flags) cudaFreeHost(h_flags);
    if (fft) fft_tables_destroy(fft);
    for (int k = 0; k < kSide; ++k) {
      if (side[k]) cudaStreamDestroy(side[k]);
      if (ev_side[k]) cudaEventDestroy(ev_side[k]);
    }
    if (ev_grid) cudaEventDestroy(ev_grid);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

wgpu_plan_request_t job_request(const wgpu_facets &f, const Job &j, int64_t force_support) {
  wgpu_plan_request_t r;
  std::memset(&r, 0, sizeof(r));
  r.width = (int64_t)j.facet.width;
  r.height = (int64_t)j.facet.height;
  r.dl = j.facet.pixel_size_x;
  r.dm = j.facet.pixel_size_y;
  r.l_shift = j.facet.l_shift;
  r.m_shift = j.facet.m_shift;
  r.epsilon = f.epsilon;
  r.w_min = j.w_min;
  r.w_max = j.w_max;
  r.n_vis = j.count;
  r.force_support = force_support;
  r.max_plane_batch = grid_plane_group();  // one gridding group per batch
  r.memory_budget_bytes = 1e15;
  return r;
}

void bind_facets(wgpu_facets *f, size_t n_rows, size_t n_chan, const double *uvw,
                 const double *freq) {
  f->release();
  auto t_bind = Clock::now();
  cudaStream_t s = f->stream;
  if (n_rows == 0 || n_chan == 0) throw Error(WGPU_ERR_INVALID, "empty visibility set");
  if (f->groups.back() > n_chan) throw Error(WGPU_ERR_INVALID, "channel group beyond n_chan");
  f->n_rows = n_rows;
  f->n_chan = n_chan;
  f->d_uvw = (double *)f->alloc(sizeof(double) * 3 * n_rows);
  f->d_freq = (double *)f->alloc(sizeof(double) * n_chan);
  f->d_vis = (float2 *)f->alloc(sizeof(float2) * n_rows * n_chan);
  f->d_vis_facet.clear();
  f->d_vis_raw = nullptr;
  f->vis_raw_floats = 0;
  f->d_sol = nullptr;
  f->sol_floats = 0;
  if (f->per_facet) {
    for (size_t i = 0; i < f->facets.size(); ++i)
      f->d_vis_facet.push_back((float2 *)f->alloc(sizeof(float2) * n_rows * n_chan));
    f->d_ant = (uint64_t *)f->alloc(sizeof(uint64_t) * 2 * n_rows);
    f->d_tof = (uint64_t *)f->alloc(sizeof(uint64_t) * n_rows);
    f->d_err = (int *)f->alloc(sizeof(int) * 4);
  }
  WGPU_CUDA(cudaMemcpyAsync(f->d_uvw, uvw, sizeof(double) * 3 * n_rows, cudaMemcpyHostToDevice, s));
  WGPU_CUDA(cudaMemcpyAsync(f->d_freq, freq, sizeof(double) * n_chan, cudaMemcpyHostToDevice, s));
  DeviceArena &arena = f->scratch;

  // jobs: group-major (job = group * n_facets + facet); w extent per group
  const size_t n_groups = f->groups.size() - 1;
  for (size_t gi = 0; gi < n_groups; ++gi) {
    const int c0 = (int)f->groups[gi], nch = (int)(f->groups[gi + 1] - f->groups[gi]);
    double w_min, w_max;
    int64_t count;
    compute_w_extent(f->d_uvw, f->d_freq + c0, nullptr, nullptr, (int64_t)n_rows, nch, false,
                     &w_min, &w_max, &count, arena.get(kSlotErr, w_extent_scratch_bytes(nch)), s);
    for (const wgpu_facet_t &fc : f->facets) {
      Job j;
      j.facet = fc;
      j.c0 = c0;
      j.nch = nch;
      j.w_min = w_min;
      j.w_max = w_max;
      j.count = count;
      f->jobs.push_back(j);
    }
  }
  // support width common to all jobs: the candidate with the lowest summed
  // cost-model time among the widths the jobs would pick on their own
  int64_t w_lo = 64, w_hi = 0;
  for (Job &j : f->jobs) {
    const wgpu_plan_t p = make_plan(job_request(*f, j, 0));
    w_lo = std::min(w_lo, p.support);
    w_hi = std::max(w_hi, p.support);
  }
  double best = 1e300;
  int64_t best_w = w_hi;
  for (int64_t w = w_lo; w <= w_hi; ++w) {
    double total = 0;
    try {
      for (Job &j : f->jobs) total += make_plan(job_request(*f, j, w)).est_seconds;
    } catch (const Error &) {
      continue;  // some job cannot reach epsilon with this width
    }
    if (total < best) {
      best = total;
      best_w = w;
    }
  }
  f->support = (int)best_w;
  for (Job &j : f->jobs) {
    j.plan = make_plan(job_request(*f, j, best_w));
    j.dp = to_dev_plan(j.plan);
    j.rstride = (int)((j.plan.width + 31) / 32 * 32);
  }

  f->bind_ms[0] = ms_since(t_bind);
  t_bind = Clock::now();
  // per job: bucketing into owned buffers, tables, work items
  f->image_elems = 0;
  for (Job &j : f->jobs) f->image_elems += j.facet.width * j.facet.height;
  f->d_images = (float *)f->alloc(sizeof(float) * f->image_elems);
  size_t img_off = 0;
  for (Job &j : f->jobs) {
    const BucketResult br = bucket_visibilities(arena, j.dp, f->d_uvw, f->d_freq + j.c0, nullptr,
                                                nullptr, (int64_t)n_rows, j.nch, false,
                                                f->d_flags, s);
    j.n_out = br.n_out;
    j.n_keys = br.n_keys;
    j.geom = (VisRecord *)f->alloc(sizeof(VisRecord) * (br.n_out + 1));
    j.work = (VisRecord *)f->alloc(sizeof(VisRecord) * (br.n_out + 1));
    j.perm = (uint32_t *)f->alloc(sizeof(uint32_t) * (br.n_out + 1));
    j.offsets = (uint32_t *)f->alloc(sizeof(uint32_t) * (br.n_keys + 1));
    WGPU_CUDA(cudaMemcpyAsync(j.geom, br.records, sizeof(VisRecord) * br.n_out,
                              cudaMemcpyDeviceToDevice, s));
    WGPU_CUDA(cudaMemcpyAsync(j.perm, br.perm, sizeof(uint32_t) * br.n_out,
                              cudaMemcpyDeviceToDevice, s));
    WGPU_CUDA(cudaMemcpyAsync(j.offsets, br.offsets, sizeof(uint32_t) * (br.n_keys + 1),
                              cudaMemcpyDeviceToDevice, s));
    j.rows_occ = copy_row_occupancy(br.rows, f->alloc(br.rows.bytes()), s);
    const int64_t npix = j.plan.width * j.plan.height;
    j.acc = (float2 *)f->alloc(sizeof(float2) * npix);
    j.nu_w = (double *)f->alloc(sizeof(double) * npix);
    launch_nu_table(j.dp, j.nu_w, s);
    j.scr = screen_table_at(f->alloc(kScreenBytesPerPixel * npix), npix);
    launch_screen_table(j.dp, j.nu_w, j.scr, s);
    j.cx = (float *)f->alloc(sizeof(float) * j.plan.width);
    j.cy = (float *)f->alloc(sizeof(float) * j.plan.height);
    j.gl = (float *)f->alloc(sizeof(float) * 2 * kCorrGlNodes);
    launch_correction_tables(j.plan, j.cx, j.cy, j.gl, s);
    j.wcorr = (float *)f->alloc(sizeof(float) * npix);
    launch_wcorr_table(j.dp, j.nu_w, j.gl, kCorrGlNodes, j.wcorr, s);
    j.img = f->d_images + img_off;
    img_off += j.facet.width * j.facet.height;
    wgpu_facets *fp = f;
    // spill slots come from the wave pool (set when the waves are packed)
    const ItemAlloc own = [fp](int which, size_t bytes) -> void * {
      return which == 3 ? nullptr : fp->alloc(bytes);
    };
    const int B = (int)j.plan.plane_batch;
    for (int p0 = 0; p0 < j.plan.n_planes; p0 += B) {
      const int nb = (int)std::min<int64_t>(B, j.plan.n_planes - p0);
      j.items.push_back(plan_grid_items(j.dp, j.offsets, p0, nb, own, s));
    }
    fft_twiddles(*f->fft, (int)j.plan.nu);
    fft_twiddles(*f->fft, (int)j.plan.nv);
    fft_twiddles(*f->fft, (int)j.plan.fft_n1);
    fft_twiddles(*f->fft, (int)j.plan.fft_n2);
    fft_prepare_rows(*f->fft, (int)j.plan.nu);
  }

  // the bucketing's bounded waits report into the flag word
  WGPU_CUDA(cudaMemcpyAsync(f->h_flags, f->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaStreamSynchronize(s));
  if (*f->h_flags != 0) {
    *f->h_flags = 0;
    WGPU_CUDA(cudaMemsetAsync(f->d_flags, 0, sizeof(unsigned), s));
    WGPU_CUDA(cudaStreamSynchronize(s));
    throw Error(WGPU_ERR_TIMEOUT, "a bounded device wait expired (bucket sort look-back)");
  }
  f->bind_ms[1] = ms_since(t_bind);
  t_bind = Clock::now();
  // waves of (job, plane batch) pairs within the plane budget
  std::vector<Slot> pending;
  for (int ji = 0; ji < (int)f->jobs.size(); ++ji) {
    const Job &j = f->jobs[ji];
    for (int b = 0; b < (int)j.items.size(); ++b) {
      Slot sl;
      sl.job = ji;
      sl.batch = b;
      sl.p0 = b * (int)j.plan.plane_batch;
      sl.nb = (int)std::min<int64_t>(j.plan.plane_batch, j.plan.n_planes - sl.p0);
      pending.push_back(sl);
    }
  }
  size_t pool_elems = 0;
  std::vector<Slot> wave;
  size_t used = 0;
  auto close_wave = [&] {
    if (wave.empty()) return;
    pool_elems = std::max(pool_elems, used);
    f->waves.push_back(wave);
    wave.clear();
    used = 0;
  };
  for (Slot sl : pending) {
    const Job &j = f->jobs[sl.job];
    const size_t pe = (size_t)sl.nb * j.plan.nu * j.plan.nv;
    const size_t re = (size_t)sl.nb * j.plan.nv * j.rstride;
    // every region starts on a 512-byte boundary: the row transforms read
    // planes with 16-byte bulk copies and vector loads
    const size_t se = (grid_spill_elems(j.dp, j.items[sl.batch]) + 63) / 64 * 64;
    if (!wave.empty() && (double)(used + pe + re + se) * sizeof(float2) > f->plane_budget)
      close_wave();
    sl.planes_off = used;
    sl.rows_off = used + pe;
    sl.spill_off = used + pe + re;
    used += pe + re + se;
    wave.push_back(sl);
  }
  close_wave();
  f->pool = (float2 *)f->alloc(sizeof(float2) * pool_elems);
  for (const auto &w : f->waves)
    for (const Slot &sl : w) f->jobs[sl.job].items[sl.batch].spill = f->pool + sl.spill_off;

  // job tables of each wave's gridding launch
  std::vector<GridJob *> d_jobs;
  std::vector<uint32_t *> d_base;
  std::vector<uint32_t> totals;
  for (const auto &w : f->waves) {
    std::vector<GridJob> hj;
    std::vector<uint32_t> hb;
    uint32_t total = 0;
    for (const Slot &sl : w) {
      const Job &j = f->jobs[sl.job];
      const WorkItems &wi = j.items[sl.batch];
      GridJob g;
      g.p = j.dp;
      g.rec = j.work;
      g.off = j.offsets;
      g.item_off = wi.item_off;
      g.desc = wi.desc;
      g.slot = wi.slot;
      g.spill = wi.spill;
      g.planes = f->pool + sl.planes_off;
      g.p_begin = sl.p0;
      g.n_batch = sl.nb;
      hj.push_back(g);
      hb.push_back(total);
      total += wi.total;
    }
    GridJob *dj = (GridJob *)f->alloc(sizeof(GridJob) * hj.size());
    uint32_t *db = (uint32_t *)f->alloc(sizeof(uint32_t) * hb.size());
    WGPU_CUDA(cudaMemcpyAsync(dj, hj.data(), sizeof(GridJob) * hj.size(), cudaMemcpyHostToDevice, s));
    WGPU_CUDA(cudaMemcpyAsync(db, hb.data(), sizeof(uint32_t) * hb.size(), cudaMemcpyHostToDevice, s));
    WGPU_CUDA(cudaStreamSynchronize(s));
    d_jobs.push_back(dj);
    d_base.push_back(db);
    totals.push_back(total);
  }

  f->bind_ms[2] = ms_since(t_bind);
  t_bind = Clock::now();
  // one graph for the whole inversion
  prepare_grid_items_multi(f->support);
  const uint64_t k0 = thread_launch_count();
  WGPU_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  try {
    for (size_t ji = 0; ji < f->jobs.size(); ++ji) {
      Job &j = f->jobs[ji];
      const int64_t n = j.n_out;
      // job = group * n_facets + facet: with per-facet corrections a job
      // restamps its facet's corrected visibilities
      const float2 *src = f->per_facet ? f->d_vis_facet[ji % f->facets.size()] : f->d_vis;
      if (n > 0) {
        restamp_channels_kernel<<<(unsigned)((n + kFacetThreads - 1) / kFacetThreads),
                                  kFacetThreads, 0, s>>>(j.geom, j.perm, src, n, j.nch,
                                                         (int)f->n_chan, j.c0, j.work);
        check_launch("restamp_channels_kernel");
      }
      WGPU_CUDA(cudaMemsetAsync(j.acc, 0, sizeof(float2) * j.plan.width * j.plan.height, s));
    }
    WGPU_CUDA(cudaMemsetAsync(f->d_images, 0, sizeof(float) * f->image_elems, s));
    for (size_t wi = 0; wi < f->waves.size(); ++wi) {
      for (const Slot &sl : f->waves[wi]) {
        const Job &j = f->jobs[sl.job];
        launch_zero_split_units(j.dp, j.items[sl.batch], sl.p0, sl.nb, f->pool + sl.planes_off, s);
      }
      launch_grid_items_multi(f->support, d_jobs[wi], d_base[wi], (int)f->waves[wi].size(),
                              totals[wi], s);
      // the FFT chains of the wave's pairs on side streams (a job's pairs
      // stay on one stream: they accumulate into the same image)
      WGPU_CUDA(cudaEventRecord(f->ev_grid, s));
      for (int k = 0; k < wgpu_facets::kSide; ++k)
        WGPU_CUDA(cudaStreamWaitEvent(f->side[k], f->ev_grid, 0));
      for (const Slot &sl : f->waves[wi]) {
        const Job &j = f->jobs[sl.job];
        cudaStream_t ss = f->side[sl.job % wgpu_facets::kSide];
        float2 *planes = f->pool + sl.planes_off, *rows = f->pool + sl.rows_off;
        launch_spill_fixup(j.dp, j.items[sl.batch], sl.p0, sl.nb, planes, ss);
        const RowSel sel = row_sel(j.rows_occ, sl.p0);
        launch_fft_rows_forward_crop(*f->fft, j.dp, planes, rows, j.rstride, sl.nb, sel,
                                     f->d_flags, ss);
        launch_fft_cols_a(*f->fft, j.dp, (int)j.plan.fft_n1, (int)j.plan.fft_n2, rows, j.rstride,
                          sl.nb, -1.0f, sel, ss);
        launch_fft_cols_b_forward_accumulate(*f->fft, j.dp, (int)j.plan.fft_n1,
                                             (int)j.plan.fft_n2, rows, j.rstride, sl.nb, sl.p0,
                                             j.scr, j.acc, sel, ss);
      }
      for (int k = 0; k < wgpu_facets::kSide; ++k) {
        WGPU_CUDA(cudaEventRecord(f->ev_side[k], f->side[k]));
        WGPU_CUDA(cudaStreamWaitEvent(s, f->ev_side[k], 0));
      }
    }
    for (Job &j : f->jobs)
      launch_finalize_add(j.dp, j.acc, j.wcorr, j.cx, j.cy, j.img, 4, s);
  } catch (...) {
    cudaGraph_t junk = nullptr;
    cudaStreamEndCapture(s, &junk);
    if (junk) cudaGraphDestroy(junk);
    throw;
  }
  WGPU_CUDA(cudaStreamEndCapture(s, &f->graph));
  WGPU_CUDA(cudaGraphInstantiate(&f->exec, f->graph, 0));
  f->graph_kernels = thread_launch_count() - k0;
  count_launch(-(int)f->graph_kernels);  // captured, not run
  f->bind_ms[3] = ms_since(t_bind);
  f->bound = true;
}

// Per-facet corrections: the uncorrected [row][chan][n_pol] visibilities and
// the facets' solution tables (one upload for all facets), then each facet's
// conjugated gains and collapse into its own buffer (the corrected inversion's
// kernel, callback_implementation.h:53-101 per facet).
void correct_facets(wgpu_facets *f, int mode, int n_pol, const float *vis,
                    const uint64_t *antenna_pairs, const uint64_t *time_offsets,
                    const float *solutions, int nparms, int64_t n_times, int64_t n_ant,
                    int polarization) {
  cudaStream_t s = f->stream;
  const size_t nv = f->n_rows * f->n_chan;
  const size_t vis_floats = 2 * nv * (size_t)n_pol;
  if (f->vis_raw_floats < vis_floats) {
    f->d_vis_raw = (float *)f->alloc(sizeof(float) * vis_floats);
    f->vis_raw_floats = vis_floats;
  }
  const size_t table_floats = 2 * (size_t)n_times * f->n_chan * (size_t)n_ant * (size_t)nparms;
  const size_t sol_floats = table_floats * f->facets.size();
  if (f->sol_floats < sol_floats) {
    f->d_sol = (float *)f->alloc(sizeof(float) * sol_floats);
    f->sol_floats = sol_floats;
  }
  WGPU_CUDA(cudaMemcpyAsync(f->d_vis_raw, vis, sizeof(float) * vis_floats,
                            cudaMemcpyHostToDevice, s));
  WGPU_CUDA(cudaMemcpyAsync(f->d_ant, antenna_pairs, sizeof(uint64_t) * 2 * f->n_rows,
                            cudaMemcpyHostToDevice, s));
  WGPU_CUDA(cudaMemcpyAsync(f->d_tof, time_offsets, sizeof(uint64_t) * f->n_rows,
                            cudaMemcpyHostToDevice, s));
  WGPU_CUDA(cudaMemcpyAsync(f->d_sol, solutions, sizeof(float) * sol_floats,
                            cudaMemcpyHostToDevice, s));
  WGPU_CUDA(cudaMemsetAsync(f->d_err, 0, sizeof(int), s));
  for (size_t i = 0; i < f->facets.size(); ++i)
    launch_apply_gains(mode, n_pol, (int64_t)f->n_rows, (int64_t)f->n_chan,
                       (const float2 *)f->d_vis_raw, f->d_ant, f->d_tof,
                       (const float2 *)(f->d_sol + i * table_floats), nparms, n_times, n_ant,
                       polarization, f->d_vis_facet[i], f->d_err, s);
  int herr = 0;
  WGPU_CUDA(cudaMemcpyAsync(&herr, f->d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaStreamSynchronize(s));
  if (herr) throw Error(WGPU_ERR_INVALID, "antenna index or time offset outside the solution table");
}

// vis == nullptr: the visibilities are already in place (per-facet buffers).
void invert_facets(wgpu_facets *f, const float *vis, bool device, float *images) {
  if (!f->bound) throw Error(WGPU_ERR_STATE, "no bound visibility set");
  cudaStream_t s = f->stream;
  cudaEvent_t e0, e1;
  WGPU_CUDA(cudaEventCreate(&e0));
  WGPU_CUDA(cudaEventCreate(&e1));
  WGPU_CUDA(cudaEventRecord(e0, s));
  if (vis)
    WGPU_CUDA(cudaMemcpyAsync(f->d_vis, vis, sizeof(float2) * f->n_rows * f->n_chan,
                              device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  WGPU_CUDA(cudaGraphLaunch(f->exec, s));
  count_launch((int)f->graph_kernels);
  if (images)
    WGPU_CUDA(cudaMemcpyAsync(images, f->d_images, sizeof(float) * f->image_elems,
                              device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaMemcpyAsync(f->h_flags, f->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaEventRecord(e1, s));
  WGPU_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  f->last_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (*f->h_flags != 0) {
    *f->h_flags = 0;
    WGPU_CUDA(cudaMemsetAsync(f->d_flags, 0, sizeof(unsigned), s));
    WGPU_CUDA(cudaStreamSynchronize(s));
    throw Error(WGPU_ERR_TIMEOUT, "a bounded device wait expired (row transform prefetch)");
  }
}

template <typename F>
int facets_guarded(F &&fn) {
  try {
    clear_failure();
    fn();
    return WGPU_OK;
  } catch (const Error &e) {
    return report_failure(e.status, e.what());
  } catch (const std::bad_alloc &) {
    return report_failure(WGPU_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception &e) {
    return report_failure(WGPU_ERR_INVALID, e.what());
  }
}

}  // namespace

extern "C" {

int wgpu_facets_create(const wgpu_facet_t *facets, size_t n_facets, const size_t *channel_groups,
                       size_t n_groups, double epsilon, double plane_budget_bytes,
                       wgpu_facets_t **out) {
  if (!facets || !channel_groups || !out || n_facets == 0 || n_groups == 0)
    return report_failure(WGPU_ERR_INVALID, "null or empty facet batch");
  if (!(epsilon > 0) || !(plane_budget_bytes >= 0))
    return report_failure(WGPU_ERR_INVALID, "invalid epsilon or plane budget");
  for (size_t i = 0; i < n_groups; ++i)
    if (channel_groups[i + 1] <= channel_groups[i])
      return report_failure(WGPU_ERR_INVALID, "channel groups must be increasing");
  for (size_t i = 0; i < n_facets; ++i)
    if (facets[i].width == 0 || facets[i].height == 0 || facets[i].width % 2 ||
        facets[i].height % 2 || !(facets[i].pixel_size_x > 0) || !(facets[i].pixel_size_y > 0))
      return report_failure(WGPU_ERR_INVALID, "facet sizes must be even and pixel sizes positive");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return report_failure(WGPU_ERR_CUDA, "no usable CUDA device");
  }
  return facets_guarded([&] {
    auto f = std::make_unique<wgpu_facets>();
    f->facets.assign(facets, facets + n_facets);
    f->groups.assign(channel_groups, channel_groups + n_groups + 1);
    f->epsilon = epsilon;
    f->plane_budget = plane_budget_bytes > 0 ? plane_budget_bytes : 40e9;
    WGPU_CUDA(cudaGetDevice(&f->device));
    WGPU_CUDA(cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking));
    for (int k = 0; k < wgpu_facets::kSide; ++k) {
      WGPU_CUDA(cudaStreamCreateWithFlags(&f->side[k], cudaStreamNonBlocking));
      WGPU_CUDA(cudaEventCreateWithFlags(&f->ev_side[k], cudaEventDisableTiming));
    }
    WGPU_CUDA(cudaEventCreateWithFlags(&f->ev_grid, cudaEventDisableTiming));
    WGPU_CUDA(cudaMalloc(&f->d_flags, sizeof(unsigned)));
    WGPU_CUDA(cudaMemset(f->d_flags, 0, sizeof(unsigned)));
    WGPU_CUDA(cudaMallocHost(&f->h_flags, sizeof(unsigned)));
    *f->h_flags = 0;
    f->fft = fft_tables_create();
    *out = f.release();
  });
}

int wgpu_facets_bind(wgpu_facets_t *f, size_t n_rows, size_t n_chan, const double *uvw,
                     const double *freq) {
  if (!f || !uvw || !freq) return report_failure(WGPU_ERR_INVALID, "null argument");
  return facets_guarded([&] {
    WGPU_CUDA(cudaSetDevice(f->device));
    f->per_facet = false;
    bind_facets(f, n_rows, n_chan, uvw, freq);
  });
}

int wgpu_facets_invert(wgpu_facets_t *f, const float *vis, float *images) {
  if (!f || !vis) return report_failure(WGPU_ERR_INVALID, "null argument");
  return facets_guarded([&] {
    if (f->per_facet)
      throw Error(WGPU_ERR_STATE, "bound with per-facet corrections: use the corrected inversion");
    invert_facets(f, vis, false, images);
  });
}

int wgpu_facets_bind_corrected(wgpu_facets_t *f, size_t n_rows, size_t n_chan, const double *uvw,
                               const double *freq) {
  if (!f || !uvw || !freq) return report_failure(WGPU_ERR_INVALID, "null argument");
  return facets_guarded([&] {
    WGPU_CUDA(cudaSetDevice(f->device));
    f->per_facet = true;
    bind_facets(f, n_rows, n_chan, uvw, freq);
  });
}

int wgpu_facets_invert_corrected(wgpu_facets_t *f, int mode, size_t n_pol, const float *vis,
                                 const uint64_t *antenna_pairs, const uint64_t *time_offsets,
                                 const float *solutions, size_t nparms, size_t n_times,
                                 size_t n_ant, int polarization, float *images) {
  if (!f || !vis || !antenna_pairs || !time_offsets || !solutions)
    return report_failure(WGPU_ERR_INVALID, "null argument");
  if (mode < WGPU_GAIN_XX || mode > WGPU_GAIN_FULL)
    return report_failure(WGPU_ERR_INVALID, "invalid gain mode");
  const size_t want = mode == WGPU_GAIN_FULL ? 4 : mode == WGPU_GAIN_2VIS_DIAGONAL ? 2 : 1;
  if (n_pol != want)
    return report_failure(WGPU_ERR_INVALID, "gain mode and n_polarizations do not match");
  if (nparms != 2 && nparms != 4) return report_failure(WGPU_ERR_INVALID, "nparms must be 2 or 4");
  if (polarization < 0 || polarization > 7)
    return report_failure(WGPU_ERR_INVALID, "invalid polarization");
  return facets_guarded([&] {
    if (!f->bound || !f->per_facet)
      throw Error(WGPU_ERR_STATE, "not bound with per-facet corrections");
    WGPU_CUDA(cudaSetDevice(f->device));
    correct_facets(f, mode, (int)n_pol, vis, antenna_pairs, time_offsets, solutions, (int)nparms,
                   (int64_t)n_times, (int64_t)n_ant, polarization);
    invert_facets(f, nullptr, false, images);
  });
}

int wgpu_facets_invert_device(wgpu_facets_t *f, const float *d_vis, float *d_images) {
  if (!f || !d_vis) return report_failure(WGPU_ERR_INVALID, "null argument");
  return facets_guarded([&] { invert_facets(f, d_vis, true, d_images); });
}

int wgpu_facets_info(const wgpu_facets_t *f, wgpu_facets_info_t *info) {
  if (!f || !info) return report_failure(WGPU_ERR_INVALID, "null argument");
  info->n_jobs = f->jobs.size();
  info->n_waves = f->waves.size();
  info->support = f->support;
  info->graph_kernels = f->graph_kernels;
  info->image_elems = f->image_elems;
  double vis = 0;
  for (const Job &j : f->jobs) vis += (double)j.n_out;
  info->job_visibilities = vis;
  info->last_ms = f->last_ms;
  for (int k = 0; k < 4; ++k) info->bind_ms[k] = f->bind_ms[k];
  return WGPU_OK;
}

int wgpu_facets_job_plan(const wgpu_facets_t *f, size_t job, wgpu_plan_t *plan) {
  if (!f || !plan) return report_failure(WGPU_ERR_INVALID, "null argument");
  if (job >= f->jobs.size()) return report_failure(WGPU_ERR_INVALID, "job index out of range");
  *plan = f->jobs[job].plan;
  return WGPU_OK;
}

void *wgpu_facets_stream(wgpu_facets_t *f) { return f ? (void *)f->stream : nullptr; }

void wgpu_facets_destroy(wgpu_facets_t *f) { delete f; }

}  // extern "C"
