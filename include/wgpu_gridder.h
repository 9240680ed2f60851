/*
 * wsclean::WGriddingGridder_Simple<NumT> on the GB300 w-gridder.
 *
 * A header-only C++ class with the interface of wgridder/gridder_simple.h
 * (WGriddingGridderBase, :19-41, and WGriddingGridder_Simple, :54-245), written
 * on the C ABI in wgpu.h.  WSClean's WGriddingMSGridder (MakeGridder,
 * wgriddingmsgridder.cpp:41-54) constructs it exactly as it constructs the
 * ducc0-backed class.  Errors from the C ABI are rethrown as
 * std::runtime_error, as the reference's MR_assert / exceptions are.
 *
 * Standalone use: define nothing; GainMode (with GetNVisibilities and
 * SelectGainMode), BandData and MsGridder are declared here.  Inside WSClean:
 * define WGPU_WITH_WSCLEAN before including, so that WSClean's own GainMode /
 * aocommon::BandData / MsGridder are used; the correction callback then reads
 * the gridder's cached h5parm solutions through VisibilityModifier, which
 * needs two read-only accessors the reference keeps private:
 *   VisibilityModifier::CachedParmResponse(ms_index)  (_cachedParmResponse)
 *   MsGridderData::OriginalMsIndex()                  (original_ms_index_)
 */
#ifndef WGPU_GRIDDER_H_
#define WGPU_GRIDDER_H_

#include <complex>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "wgpu.h"

#ifdef WGPU_WITH_WSCLEAN
/* WSClean's source root is on the include path */
#include <aocommon/banddata.h>
#include <aocommon/polarization.h>
#include "gridding/gainmode.h"
#include "gridding/msgridder.h"
#else
namespace aocommon {
class BandData;
}
namespace wsclean {
/* gridding/gainmode.h:16-31 */
enum class GainMode { kXX, kYY, kTrace, k2VisDiagonal, kFull };

/* gridding/gainmode.h:33-46 */
constexpr std::size_t GetNVisibilities(GainMode mode) {
  return mode == GainMode::k2VisDiagonal ? 2 : mode == GainMode::kFull ? 4 : 1;
}

/* gridding/gainmode.h:52-95 with the polarisation as a WGPU_POL_* value;
 * throws for the combinations the reference rejects. */
inline GainMode SelectGainMode(int polarization, std::size_t n_visibility_polarizations) {
  int mode = 0;
  if (wgpu_select_gain_mode(polarization, n_visibility_polarizations, &mode) != WGPU_OK)
    throw std::runtime_error(std::string("wgpu: ") + wgpu_last_error());
  return static_cast<GainMode>(mode);
}
class MsGridder;
}  // namespace wsclean
#endif

namespace wsclean {

/* The cached parm-response table a correction callback needs on the device:
 * complex64 solutions indexed ((t * n_chan + ch) * n_ant + ant) * nparms
 * (visibilitymodifier.h:547-551). */
struct GpuCorrectionTable {
  const std::complex<float> *solutions = nullptr;
  size_t n_times = 0;
  size_t nparms = 2;
  int polarization = WGPU_POL_STOKES_I;
};

#ifdef WGPU_WITH_WSCLEAN
/* aocommon::PolarizationEnum -> the WGPU_POL_* target of the device collapse
 * (msgridderdata.h:36-52 collapses to these). */
inline int WgpuPolarization(aocommon::PolarizationEnum polarization) {
  switch (polarization) {
    case aocommon::Polarization::StokesI: return WGPU_POL_STOKES_I;
    case aocommon::Polarization::StokesQ: return WGPU_POL_STOKES_Q;
    case aocommon::Polarization::StokesU: return WGPU_POL_STOKES_U;
    case aocommon::Polarization::StokesV: return WGPU_POL_STOKES_V;
    case aocommon::Polarization::XX: return WGPU_POL_XX;
    case aocommon::Polarization::XY: return WGPU_POL_XY;
    case aocommon::Polarization::YX: return WGPU_POL_YX;
    case aocommon::Polarization::YY: return WGPU_POL_YY;
    default:
      throw std::runtime_error("wgpu: the device collapse supports Stokes I/Q/U/V and the "
                               "linear correlations only");
  }
}

/* What MsGridderData::ApplyCorrections (msgridderdata.h:710-758) applies to the
 * rows of a correction callback, as a solution table for the device.  Returns
 * false where the reference applies no correction (not a facet, or the PSF of
 * the main image, or no h5parm solutions); fills *table with the gridder's
 * cached solutions (VisibilityModifier::_cachedParmResponse of this
 * measurement set, n_times x n_channels x n_antennas x nparms) and returns
 * true otherwise.  Throws for the two cases the device path does not cover:
 * facet beams (evaluated by EveryBeam on the host) and the direction-
 * dependent PSF (forward, then conjugated solutions). */
inline bool WgpuCorrectionTable(const MsGridder &gridder, size_t n_channels, size_t n_antennas,
                                GpuCorrectionTable *table) {
  if (!gridder.IsFacet() || gridder.GetPsfMode() == PsfMode::kSingle) return false;
  const Settings &settings = gridder.GetSettings();
  if (settings.applyFacetBeam || settings.gridWithBeam)
    throw std::runtime_error("wgpu: facet beam corrections are evaluated by EveryBeam on the "
                             "host; the GPU correction path applies h5parm solutions only");
  const VisibilityModifier &modifier = gridder.GetVisibilityModifier();
  if (!modifier.HasH5Parm()) return false;
  if (gridder.GetPsfMode() == PsfMode::kDirectionDependent)
    throw std::runtime_error("wgpu: direction-dependent PSF gridding (forward, then conjugated "
                             "solutions) is not on the device");
  const size_t ms_index = gridder.OriginalMsIndex();
  const std::vector<std::complex<float>> &solutions = modifier.CachedParmResponse(ms_index);
  table->solutions = solutions.data();
  table->nparms = modifier.NValuesPerSolution(ms_index);
  table->n_times = solutions.size() / (n_channels * n_antennas * table->nparms);
  table->polarization = WgpuPolarization(gridder.Polarization());
  return true;
}
#endif

/* gridder_simple.h:19-41 */
class WGriddingGridderBase {
 public:
  virtual ~WGriddingGridderBase() = default;
  virtual size_t ConstantMemoryUsage() const = 0;
  virtual size_t PerVisibilityMemoryUsage() const = 0;
  virtual void InitializeInversion() = 0;
  virtual void AddInversionData(size_t n_rows, size_t n_chan, const double *uvw,
                                const double *freq,
                                const std::complex<float> *vis) = 0;
  virtual void AddInversionDataWithCorrectionCallback(
      GainMode mode, size_t n_polarizations, size_t n_rows, const double *uvws,
      const double *frequencies, size_t n_channels,
      const aocommon::BandData &selected_band,
      const std::pair<size_t, size_t> *antennas,
      const std::complex<float> *visibilities, const size_t *time_offsets,
      MsGridder *gridder, size_t n_antenna) = 0;
  virtual void FinalizeImage(double multiplicationFactor) = 0;
  virtual std::vector<float> RealImage() = 0;
  virtual void InitializePrediction(const float *image_data) = 0;
  virtual void PredictVisibilities(size_t n_rows, size_t n_chan,
                                   const double *uvw, const double *freq,
                                   std::complex<float> *vis) const = 0;
};

namespace wgpu_detail {
inline void check(int status) {
  if (status != WGPU_OK)
    throw std::runtime_error(std::string("wgpu: ") + wgpu_last_error());
}
}  // namespace wgpu_detail

template <typename NumT>
class WGriddingGridder_Simple final : public WGriddingGridderBase {
  static_assert(sizeof(NumT) == 4 || sizeof(NumT) == 8, "float or double");

 public:
  static constexpr double sigma_min = 1.1;  // gridder_simple.h:57
  static constexpr double sigma_max = 2.0;  // gridder_simple.h:58

  /* gridder_simple.h:84-88; nthreads is accepted and not used (one GPU). */
  WGriddingGridder_Simple(size_t width, size_t height, size_t width_t,
                          size_t height_t, double pixelSizeX, double pixelSizeY,
                          double l_shift, double m_shift, size_t nthreads,
                          double epsilon = 1e-4, size_t verbosity = 0,
                          bool tuning = false) {
    wgpu_detail::check(wgpu_gridder_create(
        width, height, width_t, height_t, pixelSizeX, pixelSizeY, l_shift, m_shift,
        nthreads, epsilon, verbosity, tuning ? 1 : 0, (int)sizeof(NumT), &g_));
    width_ = width;
    height_ = height;
  }
  ~WGriddingGridder_Simple() override { wgpu_gridder_destroy(g_); }
  WGriddingGridder_Simple(const WGriddingGridder_Simple &) = delete;
  WGriddingGridder_Simple &operator=(const WGriddingGridder_Simple &) = delete;

  size_t ConstantMemoryUsage() const override { return wgpu_gridder_constant_memory(g_); }
  size_t PerVisibilityMemoryUsage() const override {
    return wgpu_gridder_per_visibility_memory(g_);
  }
  void InitializeInversion() override {
    wgpu_detail::check(wgpu_gridder_initialize_inversion(g_));
  }
  void AddInversionData(size_t n_rows, size_t n_chan, const double *uvw, const double *freq,
                        const std::complex<float> *vis) override {
    wgpu_detail::check(wgpu_gridder_add_inversion_data(
        g_, n_rows, n_chan, uvw, freq, reinterpret_cast<const float *>(vis)));
  }

  /* gridder_simple_implementation.h:92-110.  The device cannot call back into
   * MsGridder, so the gridder's cached solution table is read once and the
   * per-row corrections run on the GPU (kernel K7). */
  void AddInversionDataWithCorrectionCallback(
      GainMode mode, size_t n_polarizations, size_t n_rows, const double *uvws,
      const double *frequencies, size_t n_channels,
      const aocommon::BandData &selected_band,
      const std::pair<size_t, size_t> *antennas,
      const std::complex<float> *visibilities, const size_t *time_offsets,
      MsGridder *gridder, size_t n_antenna) override {
    (void)selected_band;
#ifdef WGPU_WITH_WSCLEAN
    GpuCorrectionTable table;
    if (WgpuCorrectionTable(*gridder, n_channels, n_antenna, &table)) {
      AddInversionDataWithCorrections(mode, n_polarizations, n_rows, uvws, frequencies,
                                      n_channels, antennas, visibilities, time_offsets, table,
                                      n_antenna);
    } else {
      // no correction applies; the rows are still collapsed
      // (callback_implementation.h:91-94): unit solutions, one time slot
      const size_t nparms = n_polarizations == 4 ? 4 : 2;
      std::vector<std::complex<float>> unit(n_channels * n_antenna * nparms);
      for (size_t k = 0; k < unit.size(); k += nparms) unit[k] = unit[k + nparms - 1] = 1.0f;
      const std::vector<size_t> first_slot(n_rows, 0);
      table.solutions = unit.data();
      table.n_times = 1;
      table.nparms = nparms;
      table.polarization = WgpuPolarization(gridder->Polarization());
      AddInversionDataWithCorrections(mode, n_polarizations, n_rows, uvws, frequencies,
                                      n_channels, antennas, visibilities, first_slot.data(),
                                      table, n_antenna);
    }
#else
    (void)mode; (void)n_polarizations; (void)n_rows; (void)uvws; (void)frequencies;
    (void)n_channels; (void)antennas; (void)visibilities; (void)time_offsets;
    (void)gridder; (void)n_antenna;
    throw std::runtime_error(
        "wgpu: the correction callback needs WSClean's MsGridder (build with "
        "WGPU_WITH_WSCLEAN) or AddInversionDataWithCorrections with a solution table");
#endif
  }

  /* The same with the solution table passed explicitly. */
  void AddInversionDataWithCorrections(GainMode mode, size_t n_polarizations, size_t n_rows,
                                       const double *uvws, const double *frequencies,
                                       size_t n_channels,
                                       const std::pair<size_t, size_t> *antennas,
                                       const std::complex<float> *visibilities,
                                       const size_t *time_offsets,
                                       const GpuCorrectionTable &table, size_t n_antenna) {
    static_assert(sizeof(std::pair<size_t, size_t>) == 2 * sizeof(uint64_t),
                  "antenna pairs are passed as two 64-bit indices");
    wgpu_detail::check(wgpu_gridder_add_inversion_data_corrected(
        g_, static_cast<int>(mode), n_polarizations, n_rows, uvws, frequencies, n_channels,
        reinterpret_cast<const uint64_t *>(antennas),
        reinterpret_cast<const float *>(visibilities),
        reinterpret_cast<const uint64_t *>(time_offsets),
        reinterpret_cast<const float *>(table.solutions), table.nparms, table.n_times,
        n_antenna, table.polarization));
  }

  void FinalizeImage(double multiplicationFactor) override {
    wgpu_detail::check(wgpu_gridder_finalize_image(g_, multiplicationFactor));
  }
  std::vector<float> RealImage() override {
    std::vector<float> image(width_ * height_);
    wgpu_detail::check(wgpu_gridder_real_image(g_, image.data()));
    return image;
  }
  void InitializePrediction(const float *image_data) override {
    wgpu_detail::check(wgpu_gridder_initialize_prediction(g_, image_data));
  }
  void PredictVisibilities(size_t n_rows, size_t n_chan, const double *uvw, const double *freq,
                           std::complex<float> *vis) const override {
    wgpu_detail::check(wgpu_gridder_predict_visibilities(g_, n_rows, n_chan, uvw, freq,
                                                         reinterpret_cast<float *>(vis)));
  }

  /* PredictVisibilities followed by the write-back of msgridderdata.h:180-202,
   * 943-1003 (expansion to n_polarizations correlations and the forward gains
   * of each row's antennas), on the device; vis is [row][chan][n_pol]. */
  void PredictVisibilitiesWithCorrections(GainMode mode, size_t n_polarizations,
                                          size_t n_rows, const double *uvws,
                                          const double *frequencies, size_t n_channels,
                                          const std::pair<size_t, size_t> *antennas,
                                          const size_t *time_offsets,
                                          const GpuCorrectionTable &table, size_t n_antenna,
                                          std::complex<float> *vis) const {
    static_assert(sizeof(std::pair<size_t, size_t>) == 2 * sizeof(uint64_t),
                  "antenna pairs are passed as two 64-bit indices");
    wgpu_detail::check(wgpu_gridder_predict_visibilities_corrected(
        g_, static_cast<int>(mode), n_polarizations, n_rows, uvws, frequencies, n_channels,
        reinterpret_cast<const uint64_t *>(antennas),
        reinterpret_cast<const uint64_t *>(time_offsets),
        reinterpret_cast<const float *>(table.solutions), table.nparms, table.n_times,
        n_antenna, table.polarization, reinterpret_cast<float *>(vis)));
  }

  /* WGriddingMSGridder::FinishInversion after FinalizeImage
   * (wgriddingmsgridder.cpp:273-309): RealImage resampled from the gridder's
   * size to image_width x image_height when those differ, then trimmed to
   * trim_width x trim_height, on the device. */
  std::vector<float> FinishInversion(size_t image_width, size_t image_height, size_t trim_width,
                                     size_t trim_height) {
    std::vector<float> image(trim_width * trim_height);
    wgpu_detail::check(wgpu_gridder_finish_inversion(g_, image_width, image_height, trim_width,
                                                     trim_height, image.data()));
    return image;
  }

  /* WGriddingMSGridder::StartPredict (wgriddingmsgridder.cpp:311-340): the
   * trim_width x trim_height model untrimmed, resampled to the gridder's size
   * and set as the prediction image, on the device. */
  void StartPredict(const float *model, size_t trim_width, size_t trim_height,
                    size_t image_width, size_t image_height) {
    wgpu_detail::check(wgpu_gridder_start_predict(g_, trim_width, trim_height, image_width,
                                                  image_height, model));
  }

  /* GetCollapsedVisibilities + AddInversionData on raw rows
   * (wgpu_gridder_add_inversion_rows): vis / weights [row][chan][n_pol],
   * selected [row][chan] (nullptr: all). */
  void AddInversionRows(const wgpu_imageweights_t *image_weights,
                        const wgpu_row_weighting_t &weighting, size_t n_polarizations,
                        size_t n_rows, size_t n_chan, const double *uvws,
                        const double *frequencies, const std::complex<float> *visibilities,
                        const float *weights, const std::complex<float> *model,
                        const uint8_t *selected, wgpu_weight_sums_t &sums) {
    wgpu_detail::check(wgpu_gridder_add_inversion_rows(
        g_, image_weights, &weighting, n_polarizations, n_rows, n_chan, uvws, frequencies,
        reinterpret_cast<const float *>(visibilities), weights,
        reinterpret_cast<const float *>(model), selected, &sums));
  }

  wgpu_gridder_t *handle() const { return g_; }

 private:
  wgpu_gridder_t *g_ = nullptr;
  size_t width_ = 0, height_ = 0;
};

}  // namespace wsclean

#endif  // WGPU_GRIDDER_H_
