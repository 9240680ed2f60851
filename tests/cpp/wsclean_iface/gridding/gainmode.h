// Stand-in: gridding/gainmode.h's GainMode.
#pragma once
namespace wsclean {
enum class GainMode { kXX, kYY, kTrace, k2VisDiagonal, kFull };
}  // namespace wsclean
