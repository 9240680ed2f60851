// Stand-in: aocommon::Polarization / PolarizationEnum (the values the adapter
// names).
#pragma once
namespace aocommon {
class Polarization {
 public:
  enum PolarizationEnum { StokesI, StokesQ, StokesU, StokesV, RR, RL, LR, LL, XX, XY, YX, YY };
};
using PolarizationEnum = Polarization::PolarizationEnum;
}  // namespace aocommon
