// TEST INFRASTRUCTURE ONLY.  Exposes the reference's own CalculateFFTSize
// (math/calculatefftsize.h of the reference tree, compiled from where it lies
// by oracle/Makefile's `ref` target) through a C symbol, so that the tests
// can pin the library's restatement to it.
#include <cmath>
#include <cstddef>

#include "math/calculatefftsize.h"

extern "C" void ref_calculate_fft_size(size_t size, double pixel_scale, double beam_size,
                                       size_t *minimal_size, size_t *optimal_size) {
  wsclean::CalculateFFTSize(size, pixel_scale, beam_size, *minimal_size, *optimal_size);
}
