// Stand-in: aocommon::BandData, the member the adapter's callback path uses.
#pragma once
#include <cstddef>
namespace aocommon {
class BandData {
 public:
  explicit BandData(std::size_t n_channels = 0) : n_channels_(n_channels) {}
  std::size_t ChannelCount() const { return n_channels_; }

 private:
  std::size_t n_channels_;
};
}  // namespace aocommon
