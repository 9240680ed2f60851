/*
 * wgpu -- GB300-native w-gridder, C ABI.
 *
 * This is the thin C layer between WSClean's C++ gridder interface
 * (wgridder/gridder_simple.h:19-41, WGriddingGridderBase) and the sm_103a CUDA
 * kernels.  Each entry point below names the reference method it replaces.
 * The C++ drop-in class wsclean::WGriddingGridder_Simple<NumT> in
 * include/wgpu_gridder.h is written on top of these functions.
 *
 * Conventions
 *  - All pointers are caller-owned and borrowed for the duration of the call
 *    (gridder_simple.h:106-124).  "_device" variants take device pointers and
 *    run on the gridder's CUDA stream; every other entry point takes host
 *    pointers and copies them itself.
 *  - Visibilities are interleaved complex64 (float re, float im), indexed
 *    [row * n_chan + chan]; uvw are metres [row][3]; frequencies are Hz and
 *    may be descending (gridder_simple_implementation.h:79-88).
 *  - Images passed to and from the API are row-major [x + y * width] over the
 *    UNTRIMMED width x height, exactly like RealImage()/InitializePrediction()
 *    (gridder_simple_implementation.h:147-168).
 *  - Every function returns WGPU_OK (0) or a negative status; the message of
 *    the last failure on the calling thread is returned by wgpu_last_error().
 *    There is no CPU fallback: without a usable CUDA device every compute
 *    entry point fails with WGPU_ERR_CUDA.
 */
#ifndef WGPU_H_
#define WGPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WGPU_OK 0
#define WGPU_ERR_INVALID (-1)  /* bad argument or unsupported combination */
#define WGPU_ERR_CUDA (-2)     /* CUDA runtime error / no device */
#define WGPU_ERR_NOMEM (-3)    /* device memory could not be obtained */
#define WGPU_ERR_STATE (-4)    /* call order violated (e.g. predict before init) */
#define WGPU_ERR_TIMEOUT (-5)  /* a bounded device-side wait expired */

/* Gain modes, numbered as gridding/gainmode.h:16-31 declares them. */
#define WGPU_GAIN_XX 0
#define WGPU_GAIN_YY 1
#define WGPU_GAIN_TRACE 2
#define WGPU_GAIN_2VIS_DIAGONAL 3
#define WGPU_GAIN_FULL 4

/* Polarisation selector for the 4-visibility collapse
 * (gridding/msgridderdata.h:46-50). */
#define WGPU_POL_STOKES_I 0
#define WGPU_POL_STOKES_Q 1
#define WGPU_POL_STOKES_U 2
#define WGPU_POL_STOKES_V 3
#define WGPU_POL_XX 4
#define WGPU_POL_XY 5
#define WGPU_POL_YX 6
#define WGPU_POL_YY 7
/* Further polarisations WSClean can request; wgpu_select_gain_mode tells them
 * apart as SelectGainMode does (the collapse accepts only the eight above). */
#define WGPU_POL_RR 8
#define WGPU_POL_RL 9
#define WGPU_POL_LR 10
#define WGPU_POL_LL 11
#define WGPU_POL_FULL_STOKES 12
#define WGPU_POL_INSTRUMENTAL 13
#define WGPU_POL_DIAGONAL_INSTRUMENTAL 14

/* gridding/gainmode.h:33-46 (GetNVisibilities): visibilities per sample that
 * a gain mode corrects (1, 2 or 4); 0 for a number that is no gain mode. */
size_t wgpu_gain_mode_n_visibilities(int mode);

/* gridding/gainmode.h:52-95 (SelectGainMode): the gain mode for a requested
 * polarisation (WGPU_POL_*) when n_visibility_polarizations are stored per
 * sample.  One stored polarisation: XX -> XX, YY -> YY, anything else ->
 * TRACE.  Two: Stokes I, diagonal instrumental, XX or YY -> 2VIS_DIAGONAL.
 * Four: full Stokes, instrumental, Stokes I/Q/U/V, XX or YY -> FULL.  Every
 * other combination returns WGPU_ERR_INVALID (the reference throws). */
int wgpu_select_gain_mode(int polarization, size_t n_visibility_polarizations, int *mode);

/* Message of the last failed call on this thread ("" if none). */
const char *wgpu_last_error(void);

/* Library version string. */
const char *wgpu_version(void);

/* ------------------------------------------------------------------------ */
/* Planner (host only; no device needed)                                      */
/* ------------------------------------------------------------------------ */

/* One gridding plan: grid sizes, ES kernel, w-planes.  Chosen per call from
 * the requested accuracy and the data's w range (the reference leaves this to
 * ducc0 inside ms2dirty/dirty2ms, gridder_simple.h:217-225). */
typedef struct wgpu_plan {
  int64_t width, height;  /* trimmed image */
  int64_t nu, nv;         /* padded uv grid (multiples of tile) */
  int64_t support;        /* kernel support W in cells (also in w) */
  int64_t tile;           /* uv tile edge (cells) */
  int64_t n_planes;       /* w planes (1 = no w-gridding) */
  int64_t plane_batch;    /* planes resident per pipeline step */
  int64_t fft_n1, fft_n2; /* nv = n1 * n2 column decomposition */
  double sigma;           /* oversampling of the table entry used */
  double beta;            /* ES kernel beta */
  double dl, dm, l_shift, m_shift;
  double w0, dw;          /* plane p at w0 + p * dw (wavelengths) */
  double nm1_min, nm1_max, nm1_center;
  double est_error;       /* model estimate of the relative L2 error */
  double est_seconds;     /* cost-model estimate */
} wgpu_plan_t;

typedef struct wgpu_plan_request {
  int64_t width, height;       /* trimmed image */
  double dl, dm, l_shift, m_shift;
  double epsilon;
  double w_min, w_max;         /* data w range in wavelengths */
  int64_t n_vis;               /* visibilities to grid */
  double sigma_min, sigma_max; /* 0 -> 1.1 / 2.0 (gridder_simple.h:57-58) */
  int64_t force_support;       /* >0 pins W (autotuner / tests) */
  double force_sigma;          /* >0 pins sigma */
  int64_t force_tile;          /* >0 pins the tile edge (16 or 32) */
  int64_t max_plane_batch;     /* >0 caps planes per step */
  double memory_budget_bytes;  /* >0 caps plane-batch memory */
} wgpu_plan_request_t;

int wgpu_plan_make(const wgpu_plan_request_t *request, wgpu_plan_t *plan);

/* The plans that meet the request's epsilon, lowest cost-model time first
 * (the first is wgpu_plan_make's choice): the candidates a tuning gridder
 * times.  Writes at most max_plans entries and their number to *n_plans. */
int wgpu_plan_candidates(const wgpu_plan_request_t *request, wgpu_plan_t *plans,
                         int max_plans, int *n_plans);

/* One candidate timed by a tuning gridder (tuning = 1 at creation; the
 * reference's flag selects ducc0's ms2dirty_tuning / dirty2ms_tuning,
 * gridder_simple.h:216-225, gridder_simple_implementation.h:185-194). */
typedef struct wgpu_tuning_trial {
  int64_t support;     /* kernel support W */
  double sigma;        /* oversampling */
  int64_t nu, nv;      /* grid */
  int64_t n_planes;    /* w planes */
  double est_seconds;  /* cost-model estimate */
  double measured_ms;  /* device time on the call's samples */
  int chosen;          /* 1 for the plan that was used */
} wgpu_tuning_trial_t;

/* ------------------------------------------------------------------------ */
/* Gridder instance: WGriddingGridder_Simple<NumT>                            */
/* ------------------------------------------------------------------------ */

typedef struct wgpu_gridder wgpu_gridder_t;

/* gridder_simple.h:84-88 / gridder_simple_implementation.h:32-50.
 * precision_bytes is sizeof(NumT): 4 or 8 (the type of the accumulated
 * image; the device arithmetic is FP32 with compensated accumulation either
 * way).  verbosity must be 0, 1 or 2 (the reference's MR_assert). */
int wgpu_gridder_create(size_t width, size_t height, size_t width_t,
                        size_t height_t, double pixel_size_x,
                        double pixel_size_y, double l_shift, double m_shift,
                        size_t nthreads, double epsilon, size_t verbosity,
                        int tuning, int precision_bytes,
                        wgpu_gridder_t **gridder);

void wgpu_gridder_destroy(wgpu_gridder_t *gridder);

/* gridder_simple_implementation.h:53-61 and :63-68 (same formulas). */
size_t wgpu_gridder_constant_memory(const wgpu_gridder_t *gridder);
size_t wgpu_gridder_per_visibility_memory(const wgpu_gridder_t *gridder);

/* gridder_simple_implementation.h:71-74: zero the accumulated image. */
int wgpu_gridder_initialize_inversion(wgpu_gridder_t *gridder);

/* gridder_simple_implementation.h:76-90 (AddInversionData): grid n_rows x
 * n_chan weighted, corrected visibilities and add the dirty image to the
 * accumulated image.  Visibilities equal to 0 are skipped
 * (gridder_simple.h:111). */
int wgpu_gridder_add_inversion_data(wgpu_gridder_t *gridder, size_t n_rows,
                                    size_t n_chan, const double *uvw,
                                    const double *freq, const float *vis);

/* Same, with device-resident uvw / freq / vis. */
int wgpu_gridder_add_inversion_data_device(wgpu_gridder_t *gridder,
                                           size_t n_rows, size_t n_chan,
                                           const double *d_uvw,
                                           const double *d_freq,
                                           const float *d_vis);

/* gridder_simple_implementation.h:92-110 (AddInversionDataWithCorrectionCallback)
 * with the per-row correction that VisibilityCallbackBuffer::raw performs on
 * the host (callback_implementation.h:53-101) moved onto the device: the
 * caller passes the cached solution table instead of an MsGridder pointer.
 *   vis:           [row][chan][n_pol] complex64, weighted, uncorrected
 *   antenna_pairs: [row][2] antenna indices (std::pair<size_t,size_t> layout)
 *   time_offsets:  [row] time offsets into the solution table
 *   solutions:     complex64, index ((t * n_chan + ch) * n_ant + ant) * nparms
 *                  (visibilitymodifier.h:547-551), nparms 2 (diagonal) or 4
 *   n_times:       number of time slots in the solution table
 * mode must match n_pol (1 for XX/YY/TRACE, 2 for 2VIS_DIAGONAL, 4 for FULL). */
int wgpu_gridder_add_inversion_data_corrected(
    wgpu_gridder_t *gridder, int mode, size_t n_pol, size_t n_rows,
    const double *uvw, const double *freq, size_t n_chan,
    const uint64_t *antenna_pairs, const float *vis,
    const uint64_t *time_offsets, const float *solutions, size_t nparms,
    size_t n_times, size_t n_ant, int polarization);

/* The prediction write-back of WSClean for corrected (facet / h5parm)
 * prediction: PredictVisibilities (gridder_simple_implementation.h:170-196)
 * followed by what MsGridderData::WriteCollapsedVisibilities and
 * WriteInstrumentalVisibilities do per row on the host (msgridderdata.h:180-202,
 * 943-1003): the predicted value expanded to n_pol correlations (duplicated
 * for 2, Stokes -> linear for 4 with `polarization` as in the corrected
 * inversion) and multiplied by the forward gains G1 V G2^H of the row's
 * antennas (VisibilityModifier::ApplyParmResponse, visibilitymodifier.cpp:
 * 196-228, and ApplyGain, visibilitymodifier.h:345-370), all on the device.
 * Layouts as in wgpu_gridder_add_inversion_data_corrected; the output vis is
 * [row][chan][n_pol] complex64. */
int wgpu_gridder_predict_visibilities_corrected(
    wgpu_gridder_t *gridder, int mode, size_t n_pol, size_t n_rows, const double *uvw,
    const double *freq, size_t n_chan, const uint64_t *antenna_pairs,
    const uint64_t *time_offsets, const float *solutions, size_t nparms, size_t n_times,
    size_t n_ant, int polarization, float *vis);

/* gridder_simple_implementation.h:142-145. */
int wgpu_gridder_finalize_image(wgpu_gridder_t *gridder, double factor);

/* gridder_simple_implementation.h:147-157: untrimmed width*height floats,
 * NaN outside the trimmed region. */
int wgpu_gridder_real_image(wgpu_gridder_t *gridder, float *image);

/* gridder_simple_implementation.h:159-168: untrimmed width*height model. */
int wgpu_gridder_initialize_prediction(wgpu_gridder_t *gridder,
                                       const float *image);

/* gridder_simple_implementation.h:170-196 (PredictVisibilities). */
int wgpu_gridder_predict_visibilities(wgpu_gridder_t *gridder, size_t n_rows,
                                      size_t n_chan, const double *uvw,
                                      const double *freq, float *vis);

/* Same, with device-resident uvw / freq and a device output buffer. */
int wgpu_gridder_predict_visibilities_device(wgpu_gridder_t *gridder,
                                             size_t n_rows, size_t n_chan,
                                             const double *d_uvw,
                                             const double *d_freq,
                                             float *d_vis);

/* PredictVisibilities restricted to the samples whose mask byte is non-zero
 * ([row * n_chan + chan]); the others are written as 0 and cost nothing.
 * This answers the open question in gridder_simple.h:181-182 ("how do we
 * indicate flagged visibilities that do not need to be computed?"); the
 * reference itself predicts every sample.  d_ variant: device pointers. */
int wgpu_gridder_predict_visibilities_masked(wgpu_gridder_t *gridder,
                                             size_t n_rows, size_t n_chan,
                                             const double *uvw,
                                             const double *freq,
                                             const uint8_t *mask, float *vis);
int wgpu_gridder_predict_visibilities_masked_device(
    wgpu_gridder_t *gridder, size_t n_rows, size_t n_chan, const double *d_uvw,
    const double *d_freq, const uint8_t *d_mask, float *d_vis);

/* ------------------------------------------------------------------------ */
/* Bound visibility sets: state kept on the device across major cycles        */
/* ------------------------------------------------------------------------ */

/* No counterpart in the reference, where every AddInversionData /
 * PredictVisibilities call re-plans and re-indexes its data inside ducc0.
 * WSClean's major cycles grid and predict the same rows (same uvw, same
 * flags) again and again; bind copies uvw / freq / mask to the device once,
 * plans, buckets, lays out the work items and captures the inversion and the
 * prediction pipelines in CUDA graphs.  Each later cycle only moves the
 * visibilities and replays a graph.  mask ([row * n_chan + chan], may be
 * NULL = every sample) selects the samples that take part; unselected samples
 * are predicted as 0 and ignored by the inversion.  The bound set lives until
 * unbind, a new bind or destroy.
 *   invert_bound:  adds the dirty image of `vis` to the accumulated image
 *                  (after InitializeInversion), like AddInversionData.
 *   predict_bound: predicts the bound samples from the image set by
 *                  InitializePrediction, like PredictVisibilities. */
int wgpu_gridder_bind(wgpu_gridder_t *gridder, size_t n_rows, size_t n_chan,
                      const double *uvw, const double *freq,
                      const uint8_t *mask);
int wgpu_gridder_unbind(wgpu_gridder_t *gridder);
int wgpu_gridder_invert_bound(wgpu_gridder_t *gridder, const float *vis);
int wgpu_gridder_invert_bound_device(wgpu_gridder_t *gridder,
                                     const float *d_vis);
int wgpu_gridder_predict_bound(wgpu_gridder_t *gridder, float *vis);
int wgpu_gridder_predict_bound_device(wgpu_gridder_t *gridder, float *d_vis);

/* Plan used by the last inversion/prediction call of this gridder. */
int wgpu_gridder_last_plan(const wgpu_gridder_t *gridder, wgpu_plan_t *plan);

/* Per-stage device times of the last call (milliseconds, CUDA events on the
 * gridder's stream) and the number of launches charged to each stage; names
 * are written as a ';'-separated list. */
int wgpu_gridder_last_timings(const wgpu_gridder_t *gridder, double *ms,
                              int *counts, int max_entries, char *names,
                              size_t names_len, int *n_entries);

/* Use `plan` for every following inversion/prediction call instead of
 * planning per call (NULL returns to per-call planning).  Calls whose data do
 * not fit the plan's w-planes fail with WGPU_ERR_INVALID.  Keeping one plan
 * across the major cycles of an imaging run keeps the grids comparable; it
 * has no counterpart in the reference, where ducc0 plans every call. */
int wgpu_gridder_pin_plan(wgpu_gridder_t *gridder, const wgpu_plan_t *plan);

/* Candidates timed by the last planning of a tuning gridder.  A gridder
 * created with tuning = 1 times the best few plans (wgpu_plan_candidates) on
 * the call's own samples, on this device, and uses the fastest; the choice is
 * remembered per device and request shape for the life of the process, so a
 * call that reuses it (or a gridder without tuning, or a pinned plan) reports
 * *n_trials = 0.  Writes at most max_trials entries. */
int wgpu_gridder_last_tuning(const wgpu_gridder_t *gridder, wgpu_tuning_trial_t *trials,
                             int max_trials, int *n_trials);

/* Forget every remembered tuning choice (the next tuning call times again). */
void wgpu_tuning_cache_clear(void);

/* Cap, in bytes, on the device memory of the w-plane batch that this
 * gridder's plans keep resident (0 = 40% of free device memory, at most 64 GB).
 * Lets several gridders share one GPU; no counterpart in the reference. */
int wgpu_gridder_set_plane_budget(wgpu_gridder_t *gridder, double bytes);

/* Gridder's CUDA stream (cudaStream_t), for callers that time or order work
 * around the _device entry points. */
void *wgpu_gridder_stream(wgpu_gridder_t *gridder);

/* Number of kernels this library has launched since it was loaded. */
uint64_t wgpu_kernel_launch_count(void);

/* Failure-detection self-test (no counterpart in the reference): one CTA
 * waits, with the bounded mbarrier wait the row transforms use, on a barrier
 * that nothing arrives at.  The wait must expire after timeout_ms (at most
 * 10 s) and be reported; returns WGPU_ERR_TIMEOUT in that case, WGPU_OK if
 * the wait did not expire.  The device stays usable afterwards. */
int wgpu_selftest_bounded_wait(double timeout_ms);

/* ------------------------------------------------------------------------ */
/* Bucketing pass on its own (test hook for bit-exactness)                    */
/* ------------------------------------------------------------------------ */

/* Runs the GPU bucketing pass for `plan` over host inputs and copies back, in
 * sorted order, perm (element indices row*n_chan+chan), the footprint corner
 * (iu, iv, ip), the fractions (fu, fv, fw), and the bucket offsets
 * (n_tiles*n_planes + 1 entries).  skip_zero selects inversion semantics.
 * *n_out receives the number of bucketed elements. */
int wgpu_bucket_debug(const wgpu_plan_t *plan, size_t n_rows, size_t n_chan,
                      const double *uvw, const double *freq, const float *vis,
                      int skip_zero, uint32_t *perm, int32_t *iu, int32_t *iv,
                      int32_t *ip, float *fu, float *fv, float *fw,
                      uint32_t *offsets, int64_t *n_out);

/* No counterpart in the reference (a test hook of this library).
 *
 * The same bucketing pass, returning which (w plane, grid row) pairs a
 * footprint touches: row_flags [n_planes * nv] (1 where a footprint with
 * corner (ip, iv) covers plane q = ip .. ip + W - 1 and row iv .. iv + W - 1,
 * cyclically), row_start [n_planes + 1] (first list entry of each plane) and
 * row_list [n_planes * nv] (the flagged rows as q * nv + row, by plane then
 * row; row_start[n_planes] entries are written).  Null outputs are skipped. */
int wgpu_bucket_debug_rows(const wgpu_plan_t *plan, size_t n_rows, size_t n_chan,
                           const double *uvw, const double *freq, const float *vis,
                           int skip_zero, uint8_t *row_flags, uint32_t *row_start,
                           uint32_t *row_list);

/* ------------------------------------------------------------------------ */
/* Allocation-free bucketing                                                  */
/* ------------------------------------------------------------------------ */

/* No counterpart in the reference (ducc0 does its indexing internally).
 *
 * The bucketing pass of wgpu_bucket_debug for callers that cannot allocate
 * device memory while calling into this library: for example a host that owns
 * all device memory through its own pool, or a pipeline that must not trigger
 * the device-wide synchronisation that cudaMalloc / cudaFree can cause.  The
 * caller passes device inputs and device outputs; the scratch (sort keys,
 * histograms, scan sums) lives in a static device array of
 * wgpu_bucket_noalloc_scratch_bytes() bytes (about 18 MB) that every GPU
 * loading the library holds until the process exits.  No cudaMalloc, cudaFree
 * or allocating library routine is called.
 *
 * Limits: at most WGPU_NOALLOC_MAX_VISIBILITIES samples (n_rows * n_chan),
 * WGPU_NOALLOC_MAX_CHANNELS channels and 2^26 (tile, plane) buckets; larger
 * requests fail with WGPU_ERR_INVALID.
 *
 * Outputs: d_records receives one 32-byte record per bucketed sample in sorted
 * order: float re, im (visibility times its shift phase, or the phase factor
 * for prediction), float fu, fv, fw (footprint corner minus exact position),
 * int32 iu, iv (wrapped footprint corner), int32 ip (first w plane); d_perm the
 * element index (row * n_chan + chan) of each record; d_offsets the
 * n_tiles * 4 * n_planes + 1 bucket offsets.  Size d_records and d_perm for
 * n_rows * n_chan entries; *n_out receives the number written.
 *
 * The first call on a device looks up the array's device address (with that
 * device current) and keeps it for the life of the process; make that first
 * call before any stream capture.  The kept address belongs to the device's
 * primary context: after cudaDeviceReset, or from a non-primary context on the
 * same device, the entry point must not be called again.  All calls
 * share the array and it keeps the last call's contents: calls whose work
 * overlaps on the GPU (different streams or host threads) race and must be
 * serialised by the caller.  stream may be NULL (the legacy default stream). */
#define WGPU_NOALLOC_MAX_VISIBILITIES (1 << 20)
#define WGPU_NOALLOC_MAX_CHANNELS 4096

int wgpu_bucket_noalloc(const wgpu_plan_t *plan, size_t n_rows, size_t n_chan,
                        const double *d_uvw, const double *d_freq,
                        const float *d_vis, int skip_zero, void *d_records,
                        uint32_t *d_perm, uint32_t *d_offsets, void *stream,
                        int64_t *n_out);

size_t wgpu_bucket_noalloc_scratch_bytes(void);

/* ------------------------------------------------------------------------ */
/* Request server: continuous batching of gridding requests on one GPU        */
/* ------------------------------------------------------------------------ */

/* Replaces, for this path, GriddingTaskManager / ThreadedScheduler
 * (scheduling/griddingtaskmanager.cpp:26-103, threadedscheduler.cpp:12-228),
 * which run gridding tasks on a pool of CPU threads.  Requests are queued in
 * arrival order and run by `max_active` worker slots, each with its own CUDA
 * stream, so admitted requests overlap on the device.  A request is admitted
 * when a slot is free and its estimated device memory fits what is left of
 * `device_bytes` (one that is larger than the whole budget runs alone);
 * admission is first-come first-served, except that a request whose session is
 * running waits without holding back the requests behind it.  Requests with
 * the same non-zero `session` share one gridder bound to the first request's
 * uvw / freq / mask (wgpu_gridder_bind): later requests of the session reuse
 * that device state and replay its graphs, and must carry the same geometry
 * and sample set.  A session's device memory is held until
 * wgpu_server_close_session.  Requests of one session run in submission
 * order.  Every pointer in a request must stay valid until its wait returns. */
#define WGPU_REQUEST_INVERT 1  /* vis -> image_out (FinalizeImage(image_factor)) */
#define WGPU_REQUEST_PREDICT 2 /* model -> vis_out */

typedef struct wgpu_request {
  int kind;
  uint64_t session;
  size_t width, height, width_t, height_t; /* as wgpu_gridder_create */
  double pixel_size_x, pixel_size_y, l_shift, m_shift, epsilon;
  size_t n_rows, n_chan;
  const double *uvw, *freq;
  const uint8_t *mask;  /* optional sample selection ([row * n_chan + chan]) */
  const float *vis;     /* inversion input, complex64 */
  double image_factor;  /* inversion: FinalizeImage factor */
  float *image_out;     /* inversion output, width * height */
  const float *model;   /* prediction input, width * height */
  float *vis_out;       /* prediction output, complex64 */
} wgpu_request_t;

typedef struct wgpu_server_stats {
  uint64_t completed, failed, queued, running;
  uint64_t peak_running;      /* most requests that ran at once */
  double device_bytes_in_use; /* admitted requests + resident sessions */
  double peak_device_bytes;   /* largest device_bytes_in_use */
  double visibilities;        /* n_rows * n_chan of completed requests */
  double elapsed_s;           /* first submission to last completion */
  uint64_t held_for_memory;   /* requests passed over at least once because the
                                 memory left in the budget could not take them
                                 (or an earlier request that did not fit) */
} wgpu_server_stats_t;

typedef struct wgpu_server wgpu_server_t;

/* plane_budget_bytes caps the w-plane batch of each request's plan
 * (0 = device_bytes / (2 * max_active)). */
int wgpu_server_create(double device_bytes, int max_active,
                       double plane_budget_bytes, wgpu_server_t **server);
/* Queue a request; *ticket identifies it for wgpu_server_wait. */
int wgpu_server_submit(wgpu_server_t *server, const wgpu_request_t *request,
                       uint64_t *ticket);
/* Block until the request has finished; returns its status (its message via
 * wgpu_last_error) and, if non-NULL, its latency (submission to completion)
 * and queueing time in milliseconds.  A ticket can be waited for once. */
int wgpu_server_wait(wgpu_server_t *server, uint64_t ticket,
                     double *latency_ms, double *queue_ms);
/* Release a session's gridder and device memory (WGPU_ERR_STATE while one of
 * its requests is queued or running). */
int wgpu_server_close_session(wgpu_server_t *server, uint64_t session);
int wgpu_server_stats(wgpu_server_t *server, wgpu_server_stats_t *stats);
/* Finishes the queued requests, then stops the workers and frees everything. */
void wgpu_server_destroy(wgpu_server_t *server);

/* ------------------------------------------------------------------------ */
/* Batched facets: many gridding jobs in one launch per wave                  */
/* ------------------------------------------------------------------------ */

/* Counterpart of MSGridderManager::BatchInvert with shared reads
 * (gridding/msgriddermanager.cpp:118-396): one visibility set imaged into
 * many facets (own size, pixel size and phase-centre shift, as
 * GriddingTaskFactory sets them, scheduling/griddingtaskfactory.cpp:24-34),
 * each for every output-channel group.  A job is (facet, channel group),
 * numbered group * n_facets + facet.
 *   create: channel_groups holds n_groups + 1 increasing channel boundaries.
 *   bind:   uploads uvw / freq once, plans every job with one kernel support
 *           width (the width with the lowest summed cost-model time), buckets
 *           every job, packs the jobs' 16-plane batches (planes, rows and
 *           gridding spill) into waves under plane_budget_bytes (0 = 40 GB)
 *           and captures the whole inversion
 *           in one CUDA graph: per wave, one persistent gridding launch over
 *           all the wave's jobs, then each job's FFT passes.
 *   invert: visibilities [row][chan] complex64 in, and the dirty images of
 *           all jobs out, concatenated in job order, each width * height
 *           float row-major [x + y * width] (not divided by any weight).
 * The whole visibility set and every job's sorted records stay on the device
 * until destroy; size the set to fit. */
typedef struct wgpu_facet {
  size_t width, height;           /* even */
  double pixel_size_x, pixel_size_y;
  double l_shift, m_shift;        /* facet centre relative to the phase centre */
} wgpu_facet_t;

typedef struct wgpu_facets_info {
  uint64_t n_jobs, n_waves, support, graph_kernels, image_elems;
  double job_visibilities; /* samples gridded over all jobs per inversion */
  double last_ms;          /* device time of the last inversion, incl. copies */
  double bind_ms[4];       /* host time of the last bind: upload, w extents and
                              planning; bucketing and per-job tables; waves;
                              graph capture and instantiation */
} wgpu_facets_info_t;

typedef struct wgpu_facets wgpu_facets_t;

int wgpu_facets_create(const wgpu_facet_t *facets, size_t n_facets,
                       const size_t *channel_groups, size_t n_groups,
                       double epsilon, double plane_budget_bytes,
                       wgpu_facets_t **facets_out);
int wgpu_facets_bind(wgpu_facets_t *facets, size_t n_rows, size_t n_chan,
                     const double *uvw, const double *freq);
int wgpu_facets_invert(wgpu_facets_t *facets, const float *vis, float *images);
int wgpu_facets_invert_device(wgpu_facets_t *facets, const float *d_vis,
                              float *d_images);
/* Facets with direction-dependent corrections (facet h5parm solutions, as
 * WSClean's facet gridding applies them per row through the correction
 * callback, callback_implementation.h:53-101): the batch is bound with one
 * corrected visibility buffer per facet; each inversion uploads the
 * uncorrected [row][chan][n_pol] visibilities and the facets' solution tables
 * once ([facet][t][chan][ant][nparms] complex64, layouts otherwise as in
 * wgpu_gridder_add_inversion_data_corrected), applies each facet's
 * conjugated gains and collapse on the device and runs the batch's graph. */
int wgpu_facets_bind_corrected(wgpu_facets_t *facets, size_t n_rows, size_t n_chan,
                               const double *uvw, const double *freq);
int wgpu_facets_invert_corrected(wgpu_facets_t *facets, int mode, size_t n_pol,
                                 const float *vis, const uint64_t *antenna_pairs,
                                 const uint64_t *time_offsets, const float *solutions,
                                 size_t nparms, size_t n_times, size_t n_ant, int polarization,
                                 float *images);
int wgpu_facets_info(const wgpu_facets_t *facets, wgpu_facets_info_t *info);
int wgpu_facets_job_plan(const wgpu_facets_t *facets, size_t job, wgpu_plan_t *plan);
void *wgpu_facets_stream(wgpu_facets_t *facets);
void wgpu_facets_destroy(wgpu_facets_t *facets);

/* ---- Imaging weights and per-row preparation ---------------------------
 * The imaging-weight grid of ImageWeights (structures/imageweights.h,
 * structures/imageweights.cpp) and the per-row weighting of MsGridderData
 * (CalculateWeightsImplementation + ApplyWeights + CollapseData,
 * gridding/msgridderdata.h:36-52, 515-548, 760-886) on the device, so that
 * raw measurement-set rows (visibilities, weights, selection) are weighted,
 * collapsed and gridded without a pass over them on the host. */

/* WeightMode::WeightingEnum (structures/weightmode.h:14). */
#define WGPU_WEIGHT_NATURAL 0
#define WGPU_WEIGHT_UNIFORM 1
#define WGPU_WEIGHT_BRIGGS 2

/* VisibilityWeightingMode (gridding/visibilityweightingmode.h:11-15). */
#define WGPU_VISW_NORMAL 0
#define WGPU_VISW_SQUARED 1
#define WGPU_VISW_UNIT 2

/* PsfMode (gridding/msgridderdata.h:26-32). */
#define WGPU_PSF_NONE 0
#define WGPU_PSF_SINGLE 1
#define WGPU_PSF_DIRECTION_DEPENDENT 2

/* Grid operations after FinishGridding (imageweights.cpp:149-351); the
 * meaning of wgpu_imageweights_taper's a and b per kind. */
#define WGPU_TAPER_MIN_UV 0      /* SetMinUVRange(a) */
#define WGPU_TAPER_MAX_UV 1      /* SetMaxUVRange(a) */
#define WGPU_TAPER_TUKEY 2       /* SetTukeyTaper(a = transition, b = max uv) */
#define WGPU_TAPER_TUKEY_INNER 3 /* SetTukeyInnerTaper(a = transition, b = min uv) */
#define WGPU_TAPER_EDGE 4        /* SetEdgeTaper(a) */
#define WGPU_TAPER_EDGE_TUKEY 5  /* SetEdgeTukeyTaper(a = transition, b = edge) */
#define WGPU_TAPER_GAUSSIAN 6    /* SetGaussianTaper(a = beam size, radians) */
#define WGPU_TAPER_RANK_FILTER 7 /* RankFilter(a = rank limit, b = window, <= 256) */

/* An image-weights object, like a gridder, is used by one thread at a time
 * (its float copy of the grid is refreshed on first use after a change). */
typedef struct wgpu_imageweights wgpu_imageweights_t;

/* ImageWeights(weightMode, imageWidth, imageHeight, pixelScaleX, pixelScaleY,
 * weightsAsTaper, superWeight) (imageweights.cpp:34-49): a grid of
 * width x height/2 doubles on the current device, width and height being
 * round(size / super_weight) made even.  briggs_robustness is used by
 * WGPU_WEIGHT_BRIGGS only. */
int wgpu_imageweights_create(int mode, double briggs_robustness, size_t image_width,
                             size_t image_height, double pixel_scale_x, double pixel_scale_y,
                             int weights_as_taper, double super_weight,
                             wgpu_imageweights_t **out);
void wgpu_imageweights_destroy(wgpu_imageweights_t *iw);

/* ImageWeights::Grid(MSProvider &, BandData) (imageweights.cpp:75-112) over
 * one chunk of rows: uvw [row][3] metres, freq [n_chan] Hz, weights
 * [row][chan][n_pol].  Call once per chunk, before FinishGridding. */
int wgpu_imageweights_grid(wgpu_imageweights_t *iw, size_t n_rows, size_t n_chan,
                           size_t n_pol, const double *uvw, const double *freq,
                           const float *weights);

/* Same, with device-resident uvw, freq and weights (read on the image
 * weights' stream, wgpu_imageweights_stream). */
int wgpu_imageweights_grid_device(wgpu_imageweights_t *iw, size_t n_rows, size_t n_chan,
                                  size_t n_pol, const double *d_uvw, const double *d_freq,
                                  const float *d_weights);

/* The image weights' CUDA stream (cudaStream_t). */
void *wgpu_imageweights_stream(wgpu_imageweights_t *iw);

/* FinishGridding (imageweights.cpp:114-147); a second call fails with
 * WGPU_ERR_STATE. */
int wgpu_imageweights_finish(wgpu_imageweights_t *iw);

/* One of the WGPU_TAPER_* grid operations. */
int wgpu_imageweights_taper(wgpu_imageweights_t *iw, int kind, double a, double b);

/* SetAllValues (imageweights.h:60). */
int wgpu_imageweights_set_all(wgpu_imageweights_t *iw, double value);

/* The grid: mirrored = 0 gives the width x height/2 half-plane as stored,
 * mirrored = 1 the width x height image of GetGrid (imageweights.cpp:284-300). */
int wgpu_imageweights_get(const wgpu_imageweights_t *iw, int mirrored, double *out);

/* Width(), Height() and the sum of the gridded weights. */
int wgpu_imageweights_info(const wgpu_imageweights_t *iw, size_t *width, size_t *height,
                           double *total_sum);

/* GetWeight(u, v) (imageweights.h:36) for n points in wavelengths. */
int wgpu_imageweights_sample(const wgpu_imageweights_t *iw, size_t n, const double *u,
                             const double *v, double *out);

/* What CalculateWeightsImplementation reads from the gridder's settings. */
typedef struct wgpu_row_weighting {
  int psf_mode;             /* WGPU_PSF_*: grid a point source instead of the data */
  double psf_dl, psf_dm;    /* its shift: MainImageDL/DM (single) or LShift/MShift */
  int subtract_model;       /* DoSubtractModel(): vis -= model before weighting */
  int visibility_weighting; /* WGPU_VISW_* */
  int polarization;         /* WGPU_POL_* target of the 4-correlation collapse */
} wgpu_row_weighting_t;

/* The sums ApplyWeights accumulates (msgridderdata.h:760-789); calls add to
 * them (max: the larger), so zero the struct where the reference resets
 * them (msgridderdata.h:253-259). */
typedef struct wgpu_weight_sums {
  double visibility_weight_sum;      /* VisibilityWeightSum() */
  double max_gridded_weight;         /* MaxGriddedWeight() */
  double total_weight;               /* total_weight_ */
  uint64_t gridded_visibility_count; /* GriddedVisibilityCount() */
} wgpu_weight_sums_t;

/* CalculateWeights + ApplyWeights + CollapseData for rows without
 * corrections (msgridderdata.h:515-548, 760-886), on the image weights'
 * device:
 *   vis      [row][chan][n_pol] complex64 (not read in PSF mode: may be NULL)
 *   weights  [row][chan][n_pol] visibility weights
 *   model    [row][chan][n_pol] complex64 (read when subtract_model)
 *   selected [row][chan] bytes, 0 = not gridded in this pass (NULL: all)
 * Outputs: vis_out [row][chan] complex64 (weighted, collapsed to one value),
 * weights_out [row][chan][n_pol] (the cumulative weights ApplyWeights leaves
 * in the weight buffer; may be NULL), imaging_weights_out [row][chan] (what
 * StoreImagingWeights writes; may be NULL); sums may be NULL. */
int wgpu_prepare_rows(const wgpu_imageweights_t *iw, const wgpu_row_weighting_t *rw,
                      size_t n_pol, size_t n_rows, size_t n_chan, const double *uvw,
                      const double *freq, const float *vis, const float *weights,
                      const float *model, const uint8_t *selected, float *vis_out,
                      float *weights_out, float *imaging_weights_out,
                      wgpu_weight_sums_t *sums);

/* Same on device buffers (the image weights' stream); sums are read back. */
int wgpu_prepare_rows_device(const wgpu_imageweights_t *iw, const wgpu_row_weighting_t *rw,
                             size_t n_pol, size_t n_rows, size_t n_chan, const double *d_uvw,
                             const double *d_freq, const float *d_vis, const float *d_weights,
                             const float *d_model, const uint8_t *d_selected, float *d_vis_out,
                             float *d_weights_out, float *d_imaging_weights_out,
                             wgpu_weight_sums_t *sums);

/* GetCollapsedVisibilities followed by AddInversionData for one chunk of raw
 * rows (WGriddingMSGridder::GridMeasurementSet, wgridder/wgriddingmsgridder.cpp:
 * 117-180, without corrections): the
 * rows are weighted and collapsed as in wgpu_prepare_rows, on the gridder's
 * stream, and gridded without leaving the device. */
int wgpu_gridder_add_inversion_rows(wgpu_gridder_t *gridder, const wgpu_imageweights_t *iw,
                                    const wgpu_row_weighting_t *rw, size_t n_pol,
                                    size_t n_rows, size_t n_chan, const double *uvw,
                                    const double *freq, const float *vis,
                                    const float *weights, const float *model,
                                    const uint8_t *selected, wgpu_weight_sums_t *sums);

/* GetCollapsedVisibilities with h5parm corrections followed by
 * AddInversionData (ApplyWeightsAndCorrections, msgridderdata.h:888-927,
 * through VisibilityModifier::ApplyConjugatedParmResponse,
 * visibilitymodifier.h:538-594): each raw row is weighted as in
 * wgpu_prepare_rows, the conjugated gains of its antennas are applied to its
 * correlations before ApplyWeights, and it is collapsed and gridded, all on
 * the device.  mode / n_pol, antenna_pairs, time_offsets and the solution
 * table as in wgpu_gridder_add_inversion_data_corrected.  correction_sum (may
 * be NULL) accumulates the AverageCorrection sum (averagecorrection.h:36-50)
 * of the gridded samples, with w the visibility weight of the first
 * correlation times the imaging weight:
 *   TRACE:  correction_sum[0] += |g|^2 w, g = (g2[0] conj(g1[0]) +
 *           g2[3] conj(g1[3])) / 2;
 *   others: correction_sum[0..31] += 0.5 w (a^H a + b^H b) with the
 *           Kronecker products a = G1 (x) G2 and b = G2 (x) G1, a Hermitian
 *           4 x 4 complex matrix stored row-major as (re, im) pairs (element
 *           (2i + k, 2j + l) of G1 (x) G2 is G1[i][j] G2[k][l]).  aocommon's
 *           packed HMatrix4x4 storage is not reproduced; a^H a is used where
 *           the reference's HermitianSquare order is not pinned (the two orders
 *           agree for diagonal solutions, which its known answers fix). */
int wgpu_gridder_add_inversion_rows_corrected(
    wgpu_gridder_t *gridder, const wgpu_imageweights_t *iw, const wgpu_row_weighting_t *rw,
    int mode, size_t n_pol, size_t n_rows, size_t n_chan, const double *uvw,
    const double *freq, const float *vis, const float *weights, const float *model,
    const uint8_t *selected, const uint64_t *antenna_pairs, const uint64_t *time_offsets,
    const float *solutions, size_t nparms, size_t n_times, size_t n_ant,
    wgpu_weight_sums_t *sums, double *correction_sum);

/* ---- Resampling and trimming around the boundary -------------------------
 * WGriddingMSGridder::FinishInversion / StartPredict
 * (wgridder/wgriddingmsgridder.cpp:273-340) move the image between the padded
 * image size and the inversion size of the small inversion with an FFT
 * resampler (schaapcommon's, absent from the reference tree; restated as the
 * published method: half-spectrum copy of the low frequencies, inverse, factor
 * 1 / (in_w * in_h)) and trim / untrim it around the centre. */

/* CalculateFFTSize (math/calculatefftsize.h:24-35): the Nyquist-sampled size of
 * `size` pixels of pixel_scale for a beam of beam_size (radians), and the
 * next multiple of 4 with only factors 2, 3, 5, 7 (at most size). */
int wgpu_calculate_fft_size(size_t size, double pixel_scale, double beam_size,
                            size_t *minimal_size, size_t *optimal_size);

/* The small-inversion sizes of MsGridder::CalculateOverallMetaData
 * (gridding/msgridder.cpp:42-75): when the optimal FFT size is smaller than
 * the image, the inversion size (at least 32) and its larger pixels;
 * otherwise the inputs unchanged. */
int wgpu_small_inversion_size(size_t width, size_t height, double pixel_size_x,
                              double pixel_size_y, double beam_size, size_t *inversion_width,
                              size_t *inversion_height, double *inversion_pixel_x,
                              double *inversion_pixel_y);

/* getActualTrimmedSize (wgridder/wgriddingmsgridder.cpp:243-260): the
 * gridder's trimmed size for an inversion size and image padding. */
int wgpu_actual_trimmed_size(size_t inversion_width, size_t inversion_height,
                             double image_padding, size_t *trimmed_width,
                             size_t *trimmed_height);

/* FFT resampling of a row-major in_w x in_h float image to out_w x out_h
 * (sizes 1 to 65536 whose prime factors are at most 64); non-finite input
 * pixels count as 0.  The device variant runs on `stream` (cudaStream_t, NULL
 * for the default stream). */
int wgpu_resample(const float *in, size_t in_w, size_t in_h, float *out, size_t out_w,
                  size_t out_h);
int wgpu_resample_device(const float *d_in, size_t in_w, size_t in_h, float *d_out,
                         size_t out_w, size_t out_h, void *stream);

/* FinishInversion after FinalizeImage: the gridder's image (RealImage, at the
 * inversion size = the gridder's width x height) resampled to image_width x
 * image_height when those differ, then trimmed to trim_width x trim_height
 * (centred), into `image`; all on the device. */
int wgpu_gridder_finish_inversion(wgpu_gridder_t *gridder, size_t image_width,
                                  size_t image_height, size_t trim_width, size_t trim_height,
                                  float *image);

/* StartPredict: the trim_width x trim_height model untrimmed (zero padded,
 * centred) to image_width x image_height, resampled to the gridder's width x
 * height when those differ, then InitializePrediction; all on the device. */
int wgpu_gridder_start_predict(wgpu_gridder_t *gridder, size_t trim_width, size_t trim_height,
                               size_t image_width, size_t image_height, const float *model);

#ifdef __cplusplus
}
#endif

#endif /* WGPU_H_ */
