/*
 * wsclean::GpuImageWeights -- the imaging-weight grid of WSClean's
 * ImageWeights (structures/imageweights.h) held on the GPU, over the C ABI of
 * include/wgpu.h.  The methods keep the reference's names and argument
 * meaning; Grid takes one chunk of rows (the reference reads them from an
 * MSProvider).  Header-only.
 */
#ifndef WGPU_IMAGEWEIGHTS_H_
#define WGPU_IMAGEWEIGHTS_H_

#include <stdexcept>
#include <string>
#include <vector>

#include "wgpu.h"

namespace wsclean {

class GpuImageWeights {
 public:
  /* ImageWeights(weightMode, imageWidth, imageHeight, pixelScaleX,
   * pixelScaleY, weightsAsTaper, superWeight) (imageweights.cpp:34-49);
   * mode is WGPU_WEIGHT_NATURAL / _UNIFORM / _BRIGGS. */
  GpuImageWeights(int mode, double briggs_robustness, size_t image_width, size_t image_height,
                  double pixel_scale_x, double pixel_scale_y, bool weights_as_taper,
                  double super_weight) {
    check(wgpu_imageweights_create(mode, briggs_robustness, image_width, image_height,
                                   pixel_scale_x, pixel_scale_y, weights_as_taper ? 1 : 0,
                                   super_weight, &iw_));
    check(wgpu_imageweights_info(iw_, &width_, &height_, nullptr));
  }
  ~GpuImageWeights() { wgpu_imageweights_destroy(iw_); }
  GpuImageWeights(const GpuImageWeights &) = delete;
  GpuImageWeights &operator=(const GpuImageWeights &) = delete;

  /* Grid(MSProvider &, BandData) over one chunk (imageweights.cpp:75-112). */
  void Grid(size_t n_rows, size_t n_chan, size_t n_pol, const double *uvw, const double *freq,
            const float *weights) {
    check(wgpu_imageweights_grid(iw_, n_rows, n_chan, n_pol, uvw, freq, weights));
  }
  void FinishGridding() { check(wgpu_imageweights_finish(iw_)); }

  void SetMaxUVRange(double max_uv) { taper(WGPU_TAPER_MAX_UV, max_uv, 0); }
  void SetMinUVRange(double min_uv) { taper(WGPU_TAPER_MIN_UV, min_uv, 0); }
  void SetGaussianTaper(double beam_size) { taper(WGPU_TAPER_GAUSSIAN, beam_size, 0); }
  void SetTukeyTaper(double transition, double max_uv) {
    taper(WGPU_TAPER_TUKEY, transition, max_uv);
  }
  void SetTukeyInnerTaper(double transition, double min_uv) {
    taper(WGPU_TAPER_TUKEY_INNER, transition, min_uv);
  }
  void SetEdgeTaper(double size) { taper(WGPU_TAPER_EDGE, size, 0); }
  void SetEdgeTukeyTaper(double transition, double edge) {
    taper(WGPU_TAPER_EDGE_TUKEY, transition, edge);
  }
  void RankFilter(double rank_limit, size_t window_size) {
    taper(WGPU_TAPER_RANK_FILTER, rank_limit, (double)window_size);
  }
  void SetAllValues(double value) { check(wgpu_imageweights_set_all(iw_, value)); }

  /* GetWeight (imageweights.h:36); u, v in wavelengths. */
  double GetWeight(double u, double v) const {
    double w = 0.0;
    check(wgpu_imageweights_sample(iw_, 1, &u, &v, &w));
    return w;
  }
  /* GetGrid (imageweights.cpp:284-300): width x height doubles. */
  void GetGrid(double *image) const { check(wgpu_imageweights_get(iw_, 1, image)); }

  size_t Width() const { return width_; }
  size_t Height() const { return height_; }
  const wgpu_imageweights_t *handle() const { return iw_; }

 private:
  static void check(int status) {
    if (status != WGPU_OK)
      throw std::runtime_error(std::string("wgpu: ") + wgpu_last_error());
  }
  void taper(int kind, double a, double b) { check(wgpu_imageweights_taper(iw_, kind, a, b)); }

  wgpu_imageweights_t *iw_ = nullptr;
  size_t width_ = 0, height_ = 0;
};

}  // namespace wsclean

#endif  // WGPU_IMAGEWEIGHTS_H_
