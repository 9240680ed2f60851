// Stand-in: the MsGridder / MsGridderData, Settings and VisibilityModifier
// members the adapter's correction callback reads, with the reference's names
// and signatures (gridding/msgridderdata.h:26-32, 265-296, 319;
// gridding/visibilitymodifier.h:170, 269-273), plus the two accessors the
// drop-in adds: VisibilityModifier::CachedParmResponse and
// MsGridderData::OriginalMsIndex.
#pragma once
#include <complex>
#include <cstddef>
#include <map>
#include <vector>

#include <aocommon/polarization.h>

namespace wsclean {

enum class PsfMode { kNone, kSingle, kDirectionDependent };

struct Settings {
  bool applyFacetBeam = false;
  bool gridWithBeam = false;
};

class VisibilityModifier {
 public:
  bool HasH5Parm() const { return !cached_parm_response_.empty(); }
  std::size_t NValuesPerSolution(std::size_t ms_index) const {
    return full_jones_.at(ms_index) ? 4 : 2;
  }
  // the accessor the drop-in adds (read-only view of _cachedParmResponse)
  const std::vector<std::complex<float>> &CachedParmResponse(std::size_t ms_index) const {
    return cached_parm_response_.at(ms_index);
  }
  // test set-up
  void SetSolutions(std::size_t ms_index, std::vector<std::complex<float>> solutions,
                    bool full_jones) {
    cached_parm_response_[ms_index] = std::move(solutions);
    full_jones_[ms_index] = full_jones;
  }

 private:
  std::map<std::size_t, std::vector<std::complex<float>>> cached_parm_response_;
  std::map<std::size_t, bool> full_jones_;
};

class MsGridderData {
 public:
  PsfMode GetPsfMode() const { return psf_mode_; }
  aocommon::PolarizationEnum Polarization() const { return polarization_; }
  const VisibilityModifier &GetVisibilityModifier() const { return visibility_modifier_; }
  VisibilityModifier &GetVisibilityModifier() { return visibility_modifier_; }
  bool IsFacet() const { return is_facet_; }
  void SetIsFacet(bool is_facet) { is_facet_ = is_facet; }
  const Settings &GetSettings() const { return settings_; }
  // the accessor the drop-in adds (original_ms_index_)
  std::size_t OriginalMsIndex() const { return original_ms_index_; }
  // test set-up
  Settings settings_;
  PsfMode psf_mode_ = PsfMode::kNone;
  aocommon::PolarizationEnum polarization_ = aocommon::Polarization::StokesI;
  std::size_t original_ms_index_ = 0;

 private:
  VisibilityModifier visibility_modifier_;
  bool is_facet_ = false;
};

class MsGridder : public MsGridderData {};

}  // namespace wsclean
