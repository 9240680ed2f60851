// Host check of wsclean_gb300/csrc/screen.cuh: the fixed-point w-screen
// phase of plane q, formed from the per-pixel terms (a, k, r) as the column
// passes form it, against (w0 + q dw) nu modulo one turn in extended
// precision, for random plans, pixels and plane indices up to 2^20.
//
// Usage: screen_phase_test N SEED
// Prints "cases <n> max_err_turns <e>"; exits 1 if e exceeds 6e-8 turns (the
// two FP32 roundings of the argument, 2^-26 turns each, plus the 2^-33
// rounding of a).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "screen.cuh"

int main(int argc, char **argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
  const unsigned seed = argc > 2 ? (unsigned)std::atoi(argv[2]) : 1u;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  double worst = 0.0;
  for (long i = 0; i < n; ++i) {
    // n - 1 - c_n of a wide field, the first plane's w and the plane step
    // (wavelengths), and a plane index: small ones and up to 2^20
    const double nu = -0.07 + 0.08 * u01(rng);
    const double w0 = -2.0e4 + 4.0e4 * u01(rng);
    const double dw = 0.1 + 500.0 * u01(rng);
    const int q = (i % 4 == 0) ? (int)(u01(rng) * (1 << 20)) : (int)(u01(rng) * 256);
    const wgpu::ScreenTerms t = wgpu::screen_terms(w0, dw, nu);
    const double arg2 = (double)wgpu::screen_arg2(t.a, t.k, t.r, q);
    const long double exact = ((long double)w0 + (long double)q * (long double)dw) *
                              (long double)nu;
    long double ref = exact - std::floor(exact);  // [0, 1)
    long double d = (long double)(arg2 * 0.5) - ref;
    d -= std::floor(d + 0.5L);  // nearest multiple of one turn taken off
    const double e = std::fabs((double)d);
    if (e > worst) worst = e;
  }
  std::printf("cases %ld max_err_turns %.3e\n", n, worst);
  return worst <= 6e-8 ? 0 : 1;
}
