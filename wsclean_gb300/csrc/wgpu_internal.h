// Internal declarations shared by the host orchestration and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/wgpu.h"

namespace wgpu {

constexpr double kSpeedOfLight = 299792458.0;
constexpr int kMaxSupport = 16;

// Exception carrying a C-ABI status; converted at the boundary.
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

#define WGPU_CUDA(call)                                                      \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      throw ::wgpu::Error(e_ == cudaErrorMemoryAllocation ? WGPU_ERR_NOMEM   \
                                                          : WGPU_ERR_CUDA,   \
                          std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void count_launch(int n = 1);
int sm_count();  // multiprocessors of the current device (cached per device)
uint64_t launch_count();
uint64_t thread_launch_count();  // launches issued by the calling thread

// Sets the calling thread's wgpu_last_error message; returns status.
int report_failure(int status, const std::string &msg);
void clear_failure();
void check_launch(const char *what);
// Raises (never lowers) a kernel's dynamic shared-memory cap; thread-safe.
void ensure_dynamic_smem(const void *fn, size_t bytes);

// One bucketed visibility in sorted order (32 bytes, two 128-bit words).
// For inversion (re, im) is the visibility times exp(-2 pi i theta); for
// prediction it is the phase factor exp(-2 pi i theta) itself.
struct __align__(16) VisRecord {
  float re, im;
  float fu, fv;  // footprint corner minus exact position, in cells
  float fw;      // same along w, in planes
  int32_t iu, iv;  // wrapped footprint corner
  int32_t ip;      // first w plane of the footprint
};
static_assert(sizeof(VisRecord) == 32, "record layout");

// Plan parameters as the kernels consume them.
struct DevPlan {
  int nu, nv, width, height, support, tile, ntu, ntv, n_planes;
  float beta;
  float w0f, inv_dwf;  // w0 and inv_dw rounded to float (FP32 footprint tests)
  // the rests of w0, inv_dw and nm1_center rounded to float, nm1_center
  // rounded to float, and the shifts as float pairs (float-float records)
  float w0l, inv_dwl, nm1_center_f, nm1_center_l;
  float l_shift_f, l_shift_l, m_shift_f, m_shift_l;
  double dl, dm, l_shift, m_shift, w0, dw, inv_dw, nm1_center;
};

DevPlan to_dev_plan(const wgpu_plan_t &p);

// One gridding job of a multi-job launch: its plan, bucketed records and
// offsets, the work items of its current plane batch and the planes they
// fill.
struct GridJob {
  DevPlan p;
  const VisRecord *rec;
  const uint32_t *off;
  const uint32_t *item_off;
  const uint32_t *desc;
  const int *slot;
  float2 *spill;
  float2 *planes;
  int p_begin, n_batch;
};

constexpr int kCorrGlNodes = 48;  // Gauss-Legendre nodes (positive half) of the w correction
// Grid-correction tables of a plan, computed on the device on stream s:
// cx[width] and cy[height] (1 / psihat per image column and row) and gl[2 *
// kCorrGlNodes] (nodes z_q and weights w_q phi(z_q) of the per-pixel w factor).
void launch_correction_tables(const wgpu_plan_t &plan, float *cx, float *cy, float *gl,
                              cudaStream_t s);


// ---- planner (plan.cpp) ----
wgpu_plan_t make_plan(const wgpu_plan_request_t &req);
// The plans that meet the request's epsilon, lowest cost-model time first (at
// most max_plans; the first is make_plan's choice).
std::vector<wgpu_plan_t> plan_candidates(const wgpu_plan_request_t &req, size_t max_plans);
void nm1_range(int64_t width, int64_t height, double dl, double dm,
               double l_shift, double m_shift, double *lo, double *hi);
int64_t good_fft_size(int64_t n, int64_t multiple);
void fft_decompose(int64_t n, int64_t *n1, int64_t *n2);
// ES kernel FT in cell units (FP64 Gauss-Legendre).
double es_fourier(double beta, int support, double f);
// The quadrature es_fourier sums: kEsQuadNodes nodes z of the positive half of
// [-1, 1] and their weights times the kernel, so that es_fourier(beta, W, f) =
// W * sum_i g[i] cos(pi f W z[i]).
constexpr int kEsQuadNodes = 256;
void es_quadrature(double beta, double *z, double *g);
double es_kernel(double beta, double z);

// ---- bucketing (bucket.cu) ----
// Which (w-plane, grid row) pairs some visibility footprint touches.  A row
// that no footprint touches holds zeros after gridding and is read by no
// visibility in degridding, so the row transforms skip it.  One device
// allocation of bytes() bytes:
//   corners [n_planes][nv] u8   1 where a footprint has its corner (ip, iv)
//   flags   [n_planes][nv] u8   1 where a footprint covers the row
//   counts  [n_planes]     u32  flagged rows per plane
//   start   [n_planes + 1] u32  first list entry of each plane
//   list    [sum counts]   u32  flagged rows as q * nv + row, by plane then row
struct RowOccupancy {
  uint8_t *buf = nullptr;
  int n_planes = 0;
  int nv = 0;
  static size_t r256(size_t b) { return (b + 255) / 256 * 256; }
  size_t cells() const { return (size_t)n_planes * (size_t)nv; }
  uint8_t *corners() const { return buf; }
  uint8_t *flags() const { return buf + r256(cells()); }
  uint32_t *counts() const { return (uint32_t *)(buf + 2 * r256(cells())); }
  uint32_t *start() const {
    return (uint32_t *)(buf + 2 * r256(cells()) + r256(4 * (size_t)n_planes));
  }
  uint32_t *list() const {
    return (uint32_t *)(buf + 2 * r256(cells()) + r256(4 * (size_t)n_planes) +
                        r256(4 * ((size_t)n_planes + 1)));
  }
  size_t bytes() const { return (size_t)((uint8_t *)list() - buf) + 4 * cells(); }
};

// Rows of one plane batch for the row transforms and column pass A: all rows
// when list is null; otherwise the batch's rows are the list entries
// start[0] .. start[n_batch] - 1 (entry - p_begin * nv is the row's index in
// the batch) and flags[b * nv + row] marks the rows of batch plane b.
struct RowSel {
  const uint8_t *flags = nullptr;
  const uint32_t *start = nullptr;
  const uint32_t *list = nullptr;
  int p_begin = 0;
};
inline RowSel row_sel(const RowOccupancy &o, int p_begin) {
  RowSel r;
  if (!o.buf) return r;
  r.flags = o.flags() + (size_t)p_begin * o.nv;
  r.start = o.start() + p_begin;
  r.list = o.list();
  r.p_begin = p_begin;
  return r;
}

struct BucketScratch;  // grow-only device buffers
struct BucketResult {
  VisRecord *records;   // [n_out]
  uint32_t *perm;       // [n_out] element index
  uint32_t *offsets;    // [n_keys + 1]
  int64_t n_out;
  int64_t n_keys;
  RowOccupancy rows;    // in the arena's occupancy slot
};
// Copies the occupancy data into dst (rows.bytes() bytes of device memory)
// and returns the view on the copy.
RowOccupancy copy_row_occupancy(const RowOccupancy &rows, void *dst, cudaStream_t s);
// Extents of the (non-zero when skip_zero) visibilities: w min/max in
// wavelengths and the count.  scratch8: w_extent_scratch_bytes(n_chan) bytes
// of device memory.
size_t w_extent_scratch_bytes(int64_t n_chan);
void compute_w_extent(const double *d_uvw, const double *d_freq,
                      const float *d_vis, const uint8_t *d_mask, int64_t n_rows,
                      int64_t n_chan, bool skip_zero, double *w_min,
                      double *w_max, int64_t *count, void *scratch8,
                      cudaStream_t s);

class DeviceArena;
// wait_flags: device word that an expired bounded wait of the sort is
// reported in (the caller checks it); null: checked here, WGPU_ERR_TIMEOUT.
BucketResult bucket_visibilities(DeviceArena &arena, const DevPlan &p,
                                 const double *d_uvw, const double *d_freq,
                                 const float *d_vis, const uint8_t *d_mask,
                                 int64_t n_rows, int64_t n_chan, bool skip_zero,
                                 unsigned *wait_flags, cudaStream_t s);

// Bucketing with scratch in a static device array (no device allocation).
size_t bucket_noalloc_scratch_bytes();
int64_t bucket_visibilities_noalloc(const DevPlan &p, const double *d_uvw, const double *d_freq,
                                    const float *d_vis, int64_t n_rows, int64_t n_chan,
                                    bool skip_zero, VisRecord *d_records, uint32_t *d_perm,
                                    uint32_t *d_offsets, cudaStream_t s);

// ---- gridding (grid.cu) ----
class DeviceArena;
// Work items of one plane batch (see grid.cu): scanned item offsets per
// (tile, plane group) unit and the item -> unit descriptors.
struct WorkItems {
  uint32_t *item_off = nullptr;
  uint32_t *desc = nullptr;
  uint32_t total = 0;
  int n_units = 0;
  // gridding only: spill slot of each unit (-1 for a unit without
  // visibilities) and the slots' border cells
  int *slot = nullptr;
  float2 *spill = nullptr;
  int n_slots = 0;
};
// Buffer provider for planning: which = 0 item offsets (and unit tables),
// 1 descriptors, 2 scan scratch, 3 spill slots.
using ItemAlloc = std::function<void *(int which, size_t bytes)>;
WorkItems plan_grid_items(const DevPlan &p, const uint32_t *off, int p_begin, int n_batch,
                          const ItemAlloc &alloc, cudaStream_t s);
WorkItems plan_degrid_items(const DevPlan &p, const uint32_t *off, int p_begin, int n_batch,
                            const ItemAlloc &alloc, cudaStream_t s);
void launch_zero_split_units(const DevPlan &p, const WorkItems &wi, int p_begin, int n_batch,
                             float2 *planes, cudaStream_t s);
void launch_grid_items(const DevPlan &p, const VisRecord *rec, const uint32_t *off, int p_begin,
                       int n_batch, const WorkItems &wi, float2 *planes, cudaStream_t s);
// All jobs' items in one persistent launch (items of job j start at
// d_base[j]); every job has kernel support `support`.
// float2 elements of a gridding batch's spill slots (an allocator that
// returns null for `which` 3 leaves WorkItems::spill for the caller to set).
size_t grid_spill_elems(const DevPlan &p, const WorkItems &wi);
// Adds the units' spilled border cells into the neighbouring tiles' cells;
// runs after the gridding of a plane batch (launch_grid_items does it).
void launch_spill_fixup(const DevPlan &p, const WorkItems &wi, int p_begin, int n_batch,
                        float2 *planes, cudaStream_t s);
// Sets the multi-job kernel's shared-memory cap (before a graph capture).
void prepare_grid_items_multi(int support);
void launch_grid_items_multi(int support, const GridJob *d_jobs, const uint32_t *d_base,
                             int n_jobs, uint32_t total, cudaStream_t s);
// Degridding adds into acc[s] each record's sum over the batch's planes times
// the conjugate of its phase factor (re, im).  err: device word counting
// staging waits that expired (reported by the caller as WGPU_ERR_TIMEOUT).
void launch_degrid_items(const DevPlan &p, const VisRecord *rec, const uint32_t *off,
                         int p_begin, int n_batch, const WorkItems &wi, const float2 *planes,
                         float2 *acc, unsigned *err, cudaStream_t s);
void launch_grid(DeviceArena &arena, const DevPlan &p, const VisRecord *rec,
                 const uint32_t *off, int p_begin, int n_batch, float2 *planes,
                 cudaStream_t s);
void launch_degrid(DeviceArena &arena, const DevPlan &p, const VisRecord *rec,
                   const uint32_t *off, int p_begin, int n_batch,
                   const float2 *planes, float2 *acc, unsigned *err, cudaStream_t s);
int grid_plane_group();

// ---- FFT (fft.cu) ----
struct FftTables;  // twiddles per length
const float2 *fft_twiddles(FftTables &t, int n);
FftTables *fft_tables_create();
void fft_tables_destroy(FftTables *);
int fft_row_max_length();
// Whether the row transform supports length L (multiples of 16; above 6912
// only 8192, 10240 and 12288).
bool fft_row_length_supported(int L);
// Row pass, forward: planes [B][nv][nu] -> R [B][nv][rstride] keeping the
// trimmed columns.
// Row transforms (persistent, TMA-prefetched).  err counts bounded waits that
// expired (a device word the caller checks after the call).
// Only the rows `sel` names are transformed: the other rows of R are left
// as they are (column pass A reads them as zeros through the same flags).
void launch_fft_rows_forward_crop(FftTables &t, const DevPlan &p, const float2 *planes,
                                  float2 *R, int rstride, int n_batch, const RowSel &sel,
                                  unsigned *err, cudaStream_t s);
// Row pass, backward: R -> planes (full rows), only the rows `sel` names.
void launch_fft_rows_backward_pad(FftTables &t, const DevPlan &p, const float2 *R,
                                  int rstride, float2 *planes, int n_batch, const RowSel &sel,
                                  unsigned *err, cudaStream_t s);
// Creates the row-transform tables of length L (before a graph capture).
void fft_prepare_rows(FftTables &t, int L);
// Bounded-wait self-test (fft.cu): WGPU_ERR_TIMEOUT when the wait expired.
int bounded_wait_selftest(double timeout_ms);
// Column passes (four-step split nv = n1 * n2, see fft.cu): pass A over
// strided length-n1 transforms, pass B over contiguous length-n2 transforms
// with the fused w-screen.
// Pass A with sel.flags: forward reads unflagged rows of R as zeros, backward
// writes only the flagged rows.
void launch_fft_cols_a(FftTables &t, const DevPlan &p, int n1, int n2, float2 *R,
                       int rstride, int n_batch, float sign, const RowSel &sel,
                       cudaStream_t s);
// Per-pixel w-screen terms of a plan (three planar arrays of width * height):
// the screen phase of plane q at a pixel is t = (a + q k) 2^-32 + q r turns,
// a = w0 (n - 1 - c_n) and k = dw (n - 1 - c_n) modulo one turn in 2^-32
// steps (wrapping uint32 arithmetic), r the remainder of the latter.
struct ScreenTable {
  uint32_t *a = nullptr;
  uint32_t *k = nullptr;
  float *r = nullptr;
};
constexpr size_t kScreenBytesPerPixel = 2 * sizeof(uint32_t) + sizeof(float);
// Views npix pixels of screen terms in a buffer of kScreenBytesPerPixel * npix.
ScreenTable screen_table_at(void *buf, int64_t npix);
// sel: the rows the forward row transforms wrote (read when n1 <= 1).
void launch_fft_cols_b_forward_accumulate(FftTables &t, const DevPlan &p, int n1,
                                          int n2, float2 *R, int rstride,
                                          int n_batch, int p_begin,
                                          const ScreenTable &scr, float2 *acc,
                                          const RowSel &sel, cudaStream_t s);
void launch_fft_cols_b_backward_screen(FftTables &t, const DevPlan &p, int n1,
                                       int n2, const float *img_corr,
                                       const ScreenTable &scr, float2 *R,
                                       int rstride, int n_batch, int p_begin,
                                       cudaStream_t s);

// ---- corrections (correct.cu) ----
void launch_nu_table(const DevPlan &p, double *nu_w, cudaStream_t s);
// The screen terms of plan p from its n - 1 - c_n table (FP64, once per plan).
void launch_screen_table(const DevPlan &p, const double *nu_w, const ScreenTable &scr,
                         cudaStream_t s);
// The per-pixel w correction 1 / psihat(dw (n - 1 - c_n)) of plan p, from its
// n - 1 - c_n table and the n_gl quadrature nodes gl_zw (once per plan).
void launch_wcorr_table(const DevPlan &p, const double *nu_w, const float *gl_zw, int n_gl,
                        float *wcorr, cudaStream_t s);
// tdirty * corr added into the accumulated image (float or double); corr =
// cx[x] cy[y] wcorr[pixel].
void launch_finalize_add(const DevPlan &p, const float2 *acc, const float *wcorr,
                         const float *cx, const float *cy, void *img, int precision_bytes,
                         cudaStream_t s);
// img * corr -> img_corr (prediction pre-correction).
void launch_precorrect(const DevPlan &p, const void *img, int precision_bytes,
                       const float *wcorr, const float *cx, const float *cy, float *img_corr,
                       cudaStream_t s);
void launch_scale_image(void *img, int precision_bytes, int64_t n,
                        double factor, cudaStream_t s);
void launch_restamp(const VisRecord *geom, const uint32_t *perm, const float2 *vis,
                    int64_t n, VisRecord *out, cudaStream_t s);
// vis[perm[s]] = acc[s]: the degridded sums, which the degridding already
// multiplied by the conjugate of each record's phase factor.
void launch_unpermute_predict(const uint32_t *perm, const float2 *acc, int64_t n, float2 *vis,
                              cudaStream_t s);
// Forward gains on predicted [row][chan] values -> [row][chan][n_pol]
// (prediction write-back; same layouts and error flag as launch_apply_gains).
void launch_forward_gains(int mode, int n_pol, int64_t n_rows, int64_t n_chan,
                          const float2 *vis_in, const uint64_t *ant_pairs,
                          const uint64_t *time_offsets, const float2 *sol, int nparms,
                          int64_t n_times, int64_t n_ant, int polarization, float2 *out,
                          int *err_flag, cudaStream_t s);
// ---- imaging weights and raw-row preparation (weights.cu) ----------------
// A finished imaging-weight grid as the kernels read it: width x height/2
// doubles, cell (x, y) at grid[x + y * width].
struct WeightGridView {
  const double *grid;
  const float *gridf;  // the same values as float (what the row weighting samples)
  int64_t width, height;
  double psx, psy;
};
WeightGridView imageweights_view(const wgpu_imageweights_t *iw);

// Per-call settings of the row preparation (the PSF shift's n term is formed
// on the device, rounded like the host expression).
struct RowWeighting {
  int psf_mode, subtract_model, visibility_weighting, polarization;
  double dl, dm;
};
RowWeighting row_weighting(const wgpu_row_weighting_t &rw);

// Device-side accumulators of the weight sums (zeroed by the caller).
struct WeightSumsDev {
  double visibility_weight_sum;
  double total_weight;
  unsigned long long max_bits;  // bits of the largest positive weight (double)
  unsigned long long count;
  double correction;  // TRACE correction sum (corrected rows)
  // matrix correction sum of the other modes (corrected rows): the Hermitian
  // 4 x 4 matrix's diagonal (0,0) (1,1) (2,2) (3,3), then the real and
  // imaginary parts of (0,1) (0,2) (0,3) (1,2) (1,3) (2,3)
  double matrix[16];
};

// Cached parm-response table of a corrected raw-row chunk (layouts as in
// wgpu_gridder_add_inversion_data_corrected); err is a device flag set for a
// row whose antenna or time index is outside the table.
struct GainTable {
  const float2 *sol = nullptr;
  const uint64_t *ant = nullptr;
  const uint64_t *tof = nullptr;
  int nparms = 2, mode = 0;
  int64_t n_times = 0, n_ant = 0;
  int *err = nullptr;
  bool sum_matrix = false;  // accumulate the matrix correction sum (modes but TRACE)
};
void add_weight_sums(const WeightSumsDev &d, wgpu_weight_sums_t *sums);

// Work buffer (bytes) of launch_weight_grid / launch_prepare_rows for a chunk
// of n_rows x n_chan samples.
size_t pass_work_bytes(int64_t n_rows, int64_t n_chan);

// ImageWeights::Grid over n_rows x n_chan samples into grid / total.
void launch_weight_grid(const WeightGridView &g, double *grid, double *total, int as_taper,
                        int64_t n_rows, int64_t n_chan, int n_pol, const double *uvw,
                        const double *freq, const float *weights, void *work, cudaStream_t s);

// CalculateWeights + ApplyWeights + CollapseData for n_rows x n_chan samples.
void launch_prepare_rows(const WeightGridView &g, const RowWeighting &rw, int n_pol,
                         int64_t n_rows, int64_t n_chan, const double *uvw, const double *freq,
                         const float2 *vis, const float *weights, const float2 *model,
                         const uint8_t *selected, float2 *vis_out, float *weights_out,
                         float *imaging_out, WeightSumsDev *sums, void *work, cudaStream_t s,
                         const GainTable *gains = nullptr);

// ---- resampling and trimming (resample.cu) ---------------------------------
size_t resample_work_bytes(int64_t in_w, int64_t in_h, int64_t out_w, int64_t out_h);
// FFT resampling of a row-major float image (non-finite pixels count as 0).
void resample_device(const float *in, int64_t in_w, int64_t in_h, float *out, int64_t out_w,
                     int64_t out_h, void *work, cudaStream_t s);
// The centred out_w x out_h window of an in_w x in_h image, and its inverse
// (zero outside the window).
void launch_trim(const float *in, int64_t in_w, int64_t in_h, float *out, int64_t out_w,
                 int64_t out_h, cudaStream_t s);
void launch_untrim(const float *in, int64_t in_w, int64_t in_h, float *out, int64_t out_w,
                   int64_t out_h, cudaStream_t s);

void launch_apply_gains(int mode, int n_pol, int64_t n_rows, int64_t n_chan,
                        const float2 *vis_in, const uint64_t *ant_pairs,
                        const uint64_t *time_offsets, const float2 *sol,
                        int nparms, int64_t n_times, int64_t n_ant,
                        int polarization, float2 *out, int *err_flag,
                        cudaStream_t s);

// Grow-only device allocations keyed by slot.
class DeviceArena {
 public:
  DeviceArena() = default;
  ~DeviceArena();
  DeviceArena(const DeviceArena &) = delete;
  DeviceArena &operator=(const DeviceArena &) = delete;
  void *get(int slot, size_t bytes);
  size_t total() const;
  void release();
  void release(int slot);  // frees one slot (the next get allocates it again)

 private:
  static constexpr int kSlots = 48;
  void *ptr_[kSlots] = {};
  size_t size_[kSlots] = {};
};

enum ArenaSlot {
  kSlotKeys = 0,
  kSlotKeysAlt,
  kSlotVals,
  kSlotValsAlt,
  kSlotHist,
  kSlotScanTmp,
  kSlotRecords,
  kSlotOffsets,
  kSlotExtent,
  kSlotPlanes,
  kSlotRows,
  kSlotNuW,
  kSlotAcc,
  kSlotCorrX,
  kSlotCorrY,
  kSlotGl,
  kSlotVisAcc,
  kSlotUvw,
  kSlotFreq,
  kSlotVis,
  kSlotGainVis,
  kSlotAnt,
  kSlotTimes,
  kSlotSol,
  kSlotImgCorr,
  kSlotErr,
  kSlotOutVis,
  kSlotItems,
  kSlotCounter,
  kSlotItemDesc,
  kSlotSpill,
  kSlotRowOcc,
  kSlotUvwF32,
  kSlotImgIO,
  kSlotRowWeights,  // raw-row preparation: visibility weights,
  kSlotRowModel,    // model visibilities,
  kSlotRowSel,      // selection bytes,
  kSlotRowSums,     // the device-side weight sums
  kSlotRowWork,     // and the two-pass work buffer
  kSlotResampleWork,  // resampling around the boundary: FFT work images,
  kSlotResampleOut,   // the image at the padded image size,
  kSlotResampleTrim,  // and at the trimmed size
  kSlotCorner,        // bucketing: footprint corner within the tile, per sample
  kSlotScreen,        // per-pixel w-screen terms of the current plan
  kSlotWCorr,         // per-pixel w correction of the current plan
};

// Exclusive scan of n uint32 values in place (device), returning the total.
void exclusive_scan_u32(DeviceArena &arena, uint32_t *d, int64_t n,
                        cudaStream_t s);
// Same with caller-provided scratch of exclusive_scan_scratch_words(n) words.
int64_t exclusive_scan_scratch_words(int64_t n);
void exclusive_scan_u32_scratch(uint32_t *d, int64_t n, uint32_t *tmp,
                                cudaStream_t s);

}  // namespace wgpu
