/*
 * wgpu oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU (FP64) restatements used to check the GPU w-gridder.  Nothing in the
 * product links or calls this code; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py use it, as the checker.
 *
 * Parity status:
 *  - Direct Fourier transform: restates gridding/directmsgridder.cpp (the
 *    reference's own exact transform).  The reference file cannot be compiled
 *    here (it needs aocommon, casacore and the MsGridder stack), so the
 *    restatement is pinned by analytic known-answer tests (point sources on
 *    pixel centres, constant visibilities) written against the conventions of
 *    directmsgridder.cpp:56-132,205-229.
 *  - W-gridder: the reference's arithmetic lives in ducc0 (called from
 *    wgridder/gridder_simple.h:217-225), which is absent from the reference
 *    tree.  The FP64 CPU w-gridder below follows the published method (Arras et
 *    al. 2021; Ye et al. 2021) with the same flags WSClean passes; its parity
 *    with ducc0 itself is UNPINNED.  It is checked against the DFT.
 *  - Gains and polarisation collapse: restate gridding/visibilitymodifier.h:
 *    378-401,538-594 and gridding/msgridderdata.h:36-52, pinned by the
 *    known-answer constants of tests/gridding/tvisibilitymodifier.cpp.
 */
#ifndef WGPU_ORACLE_H_
#define WGPU_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Direct FT inversion (directmsgridder.cpp:92-132): for each selected trimmed
 * pixel p = x + y*width, out[i] = sum_k Re(V_k exp(-2 pi i (u l + v m + w (n-1))))
 * with l = (width/2 - x) dl + l_shift, m = (y - height/2) dm + m_shift and
 * n-1 := 0 beyond the horizon (directmsgridder.cpp:205-229).  uvw in metres,
 * freq in Hz, vis interleaved complex64 [row][chan].  No 1/ImageWeight. */
void oracle_dft_invert(size_t n_rows, size_t n_chan, const double *uvw,
                       const double *freq, const float *vis, size_t width,
                       size_t height, double dl, double dm, double l_shift,
                       double m_shift, const int64_t *pixels, size_t n_pixels,
                       int n_threads, double *out);

/* Adjoint of oracle_dft_invert (prediction): for selected visibility
 * indices e = row*n_chan + chan, out[2i..2i+1] = sum_p I_p exp(+2 pi i (...)).
 * image is width*height doubles, row-major [x + y*width]. */
void oracle_dft_predict(size_t n_rows, size_t n_chan, const double *uvw,
                        const double *freq, const double *image, size_t width,
                        size_t height, double dl, double dm, double l_shift,
                        double m_shift, const int64_t *vis_index, size_t n_sel,
                        int n_threads, double *out);

/* Parameters of one gridding plan (all produced by the product's planner). */
typedef struct {
  int64_t width, height;   /* trimmed image */
  int64_t nu, nv;          /* padded grid */
  int64_t support;         /* W */
  int64_t tile;            /* uv tile edge in cells */
  int64_t n_planes;        /* w planes */
  double beta;             /* ES kernel beta */
  double dl, dm, l_shift, m_shift;
  double w0, dw;           /* plane p sits at w0 + p dw (lambda) */
  double nm1_center;       /* c_n: centre of the image's n-1 range */
} OraclePlan;

/* Bucketing reference: for every included element (inversion: vis != 0;
 * prediction: all) computes the integer footprint corner, fractions and key
 * exactly as the GPU pass defines them, then orders the elements by (key,
 * footprint corner inside the tile as (iv mod tile) * tile + iu mod tile,
 * element index).
 * Outputs (n_out elements): perm[s] = element index, key[s], iu/iv/ip, fu/fv/fw.
 * offsets has n_tiles*n_planes+1 entries.  Returns n_out. */
int64_t oracle_bucket(const OraclePlan *plan, size_t n_rows, size_t n_chan,
                      const double *uvw, const double *freq, const float *vis,
                      int skip_zero, uint32_t *perm, int64_t *key, int32_t *iu,
                      int32_t *iv, int32_t *ip, float *fu, float *fv,
                      float *fw, int64_t *offsets);

/* FP64 CPU w-gridder, inversion: dirty[x + y*width] (trimmed, DFT
 * orientation) = sum over included vis, computed by gridding + FFT + w-screen +
 * correction.  Returns 0 on success. */
int oracle_wgrid_invert(const OraclePlan *plan, size_t n_rows, size_t n_chan,
                        const double *uvw, const double *freq, const float *vis,
                        int n_threads, double *dirty);

/* FP64 CPU w-gridder, prediction (adjoint): vis_out interleaved complex
 * doubles [row][chan]. */
int oracle_wgrid_predict(const OraclePlan *plan, size_t n_rows, size_t n_chan,
                         const double *uvw, const double *freq,
                         const double *image, int n_threads, double *vis_out);

/* Timing helper for the CPU baseline: grids (no FFT) the included visibilities
 * onto the planes they touch, in FP64, and returns seconds spent; and runs
 * plane_fraction (0 < f <= 1) of one inversion plane pass (the row FFTs and
 * cropped column FFTs + screen of that fraction of rows and columns),
 * returning its seconds in *plane_seconds. */
double oracle_wgrid_time_parts(const OraclePlan *plan, size_t n_rows,
                               size_t n_chan, const double *uvw,
                               const double *freq, const float *vis,
                               int n_threads, double plane_fraction,
                               double *plane_seconds);

/* The prediction's counterpart: interpolates the samples with vis != 0 from
 * the planes they touch (no FFT), in FP64, returning seconds spent; and runs
 * plane_fraction of one prediction plane pass (screen, inverse column and row
 * FFTs), returning its seconds in *plane_seconds. */
double oracle_wgrid_time_predict_parts(const OraclePlan *plan, size_t n_rows,
                                       size_t n_chan, const double *uvw,
                                       const double *freq, const float *vis,
                                       int n_threads, double plane_fraction,
                                       double *plane_seconds);

/* AverageCorrection::Add, matrix form (averagecorrection.h:36-50): adds
 * 0.5 w ((G1 (x) G2)^H (G1 (x) G2) + (G2 (x) G1)^H (G2 (x) G1)) to sum, a 4 x 4
 * complex matrix stored row-major as 32 doubles (re, im).  g1, g2: 2 x 2
 * gains, row-major, interleaved complex64.  aocommon's HermitianSquare is
 * absent from the reference tree; M^H M is used (for diagonal gains both
 * orders agree, which the reference's known answers pin). */
void oracle_correction_matrix_add(const float *g1, const float *g2, double w, double *sum);

/* ES kernel value at z in [-1,1] and its continuous FT in cell units. */
double oracle_es_kernel(double beta, double z);
double oracle_es_fourier(double beta, int support, double f);

/* Gains (visibilitymodifier.h:378-401) applied in conjugate for every row and
 * channel, followed by the polarisation collapse (msgridderdata.h:36-52).
 * mode: 0 kXX, 1 kYY, 2 kTrace, 3 k2VisDiagonal, 4 kFull (gainmode.h:16-31).
 * vis_in: [row][chan][n_pol] complex64; solutions: complex64 with the cached
 * parm-response layout ((t*n_chan + ch)*n_ant + ant)*nparms; out: collapsed
 * [row][chan] complex64.  polarization (4-pol collapse): 0 StokesI, 1 Q, 2 U,
 * 3 V, 4 XX, 5 XY, 6 YX, 7 YY.  Returns 0 on success, -1 on a bad combination. */
/* Prediction write-back: predicted [row][chan] complex64 values expanded to
 * n_pol correlations (1: as is; 2: duplicated, msgridderdata.h:58-62; 4:
 * Stokes -> linear, the inverse of the collapse above) and multiplied by the
 * forward gains (visibilitymodifier.h:345-370 through visibilitymodifier.cpp:
 * 196-228).  out: [row][chan][n_pol] complex64.  Same layouts and return
 * values as oracle_apply_gains. */
int oracle_forward_gains(int mode, size_t n_pol, size_t n_rows, size_t n_chan,
                         const float *vis_in, const uint64_t *antenna_pairs,
                         const uint64_t *time_offsets, const float *solutions,
                         size_t nparms, size_t n_ant, int polarization, float *out);
int oracle_apply_gains(int mode, size_t n_pol, size_t n_rows, size_t n_chan,
                       const float *vis_in, const uint64_t *antenna_pairs,
                       const uint64_t *time_offsets, const float *solutions,
                       size_t nparms, size_t n_ant, int polarization,
                       float *out);

/* Single-visibility-group gain application used by the known-answer tests. */
void oracle_apply_conjugated_gain(int mode, float *vis, const float *g1,
                                  const float *g2);
void oracle_apply_gain(int mode, float *vis, const float *g1, const float *g2);

/* ---- Imaging weights and raw-row weighting --------------------------------
 * ImageWeights (structures/imageweights.h, structures/imageweights.cpp) and
 * MsGridderData's CalculateWeightsImplementation + ApplyWeights + CollapseData
 * (gridding/msgridderdata.h:36-52, 760-886), restated in serial loops in the
 * reference's order.  Parity status: pinned by reading the reference source
 * (it needs aocommon, which the reference tree does not contain, so it cannot
 * be built here) and by the pure-Python known-answer restatement in the
 * tests.  The wavelength of a channel is 299792458 / frequency in double; the
 * 4-correlation collapse is the convention of collapse4 above (unpinned).
 * The grid is width x height/2 doubles, cell (x, y) at [x + y * width]. */

/* imageweights.cpp:34-49: the grid size after the super weight. */
void oracle_weights_dims(size_t image_width, size_t image_height, double super_weight,
                         int64_t *width, int64_t *height);
/* Grid(MSProvider &, BandData) (imageweights.cpp:75-112) over one chunk;
 * returns the weight it added to the total. */
double oracle_weights_grid(double *grid, int64_t width, int64_t height, double psx, double psy,
                           int as_taper, size_t n_rows, size_t n_chan, size_t n_pol,
                           const double *uvw, const double *freq, const float *weights);
/* FinishGridding (imageweights.cpp:114-147); mode 0 natural, 1 uniform,
 * 2 Briggs. */
void oracle_weights_finish(double *grid, int64_t width, int64_t height, int mode,
                           double robustness, double total_sum);
/* The WGPU_TAPER_* operations (imageweights.cpp:149-351), same a / b. */
void oracle_weights_taper(double *grid, int64_t width, int64_t height, double psx, double psy,
                          int kind, double a, double b);
/* GetGrid (imageweights.cpp:284-300): width x height image. */
void oracle_weights_mirror(const double *grid, int64_t width, int64_t height, double *image);
/* GetWeight (imageweights.h:36, 98-106) for n points. */
void oracle_weights_sample(const double *grid, int64_t width, int64_t height, double psx,
                           double psy, size_t n, const double *u, const double *v, double *out);
/* One chunk of raw rows: vis / model [row][chan][n_pol] complex64 (vis unused
 * in PSF mode, model unused unless subtract_model), weights [row][chan][n_pol],
 * selected [row][chan] (NULL: all).  Outputs vis_out [row][chan], weights_out
 * [row][chan][n_pol], imaging_out [row][chan]; sums[0..3] += visibility weight
 * sum, max gridded weight (max), total weight, gridded count. */
void oracle_prepare_rows(const double *grid, int64_t width, int64_t height, double psx,
                         double psy, int psf_mode, double psf_dl, double psf_dm,
                         int subtract_model, int visibility_weighting, int polarization,
                         size_t n_pol, size_t n_rows, size_t n_chan, const double *uvw,
                         const double *freq, const float *vis, const float *weights,
                         const float *model, const uint8_t *selected, float *vis_out,
                         float *weights_out, float *imaging_out, double *sums);

/* The same with h5parm corrections: the conjugated gains of each row's
 * antennas applied to its correlations between the weighting and
 * ApplyWeights (msgridderdata.h:888-927, visibilitymodifier.h:538-594);
 * layouts as oracle_apply_gains.  correction_sum holds 33 doubles: for TRACE
 * (mode 2) correction_sum[0] += |g|^2 w iw with g = (g2[0] conj(g1[0]) +
 * g2[3] conj(g1[3])) / 2 (averagecorrection.h:36-50, 104-118); for the other
 * modes correction_sum[1..32] accumulates the matrix sum of
 * oracle_correction_matrix_add with weight w iw. */
void oracle_prepare_rows_corrected(const double *grid, int64_t width, int64_t height, double psx,
                                   double psy, int psf_mode, double psf_dl, double psf_dm,
                                   int subtract_model, int visibility_weighting, int polarization,
                                   size_t n_pol, size_t n_rows, size_t n_chan, const double *uvw,
                                   const double *freq, const float *vis, const float *weights,
                                   const float *model, const uint8_t *selected, float *vis_out,
                                   float *weights_out, float *imaging_out, double *sums, int mode,
                                   const uint64_t *antenna_pairs, const uint64_t *time_offsets,
                                   const float *solutions, size_t nparms, size_t n_ant,
                                   double *correction_sum);

#ifdef __cplusplus
}
#endif

#endif
