// Host check of wsclean_gb300/csrc/record_ff.cuh: whenever ff::decide says the
// float-float fractions and phase argument are decided, they must equal the
// FP64 chains of the record kernel bit for bit.  Built with
// -ffp-contract=off so that the FP64 reference rounds every step as the
// kernel's explicit __dmul_rn / __dsub_rn do.
//
// Usage: record_ff_test N_RANDOM N_EDGE SEED
// Prints: "random <n> decided <k> mismatches <m>" and the same for the edge
// cases; exits 1 on any mismatch.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "record_ff.cuh"

using wgpu::ff::Pair;
using wgpu::ff::split;

namespace {

struct Case {
  double u, v, w;        // metres
  double su, sv, sw;     // per-channel scales (cells per metre, wavelengths per metre)
  double w0, inv_dw, c;  // plan
  double ls, ms;         // l and m shift (0: no shift)
  int support, n_planes;
};

struct Ref {
  int iu0, iv0, ip;
  float fu, fv, fw, arg;
};

Ref reference(const Case &k) {
  Ref r;
  const double half = 0.5 * k.support;
  const double U = k.u * k.su, V = k.v * k.sv;
  r.iu0 = (int)std::ceil(U - half);
  r.iv0 = (int)std::ceil(V - half);
  r.fu = (float)((double)r.iu0 - U);
  r.fv = (float)((double)r.iv0 - V);
  const double wl = k.w * k.sw;
  if (k.n_planes > 1) {
    const double pw = (wl - k.w0) * k.inv_dw;
    double ip0 = std::ceil(pw - half);
    const double ip_max = (double)(k.n_planes - k.support);
    if (ip0 < 0.0) ip0 = 0.0;
    if (ip0 > ip_max) ip0 = ip_max;
    r.ip = (int)ip0;
    r.fw = (float)(ip0 - pw);
  } else {
    r.ip = 0;
    r.fw = 0.0f;
  }
  double t = wl * k.c;
  if (k.ls != 0.0 || k.ms != 0.0) t = ((k.u * k.sw) * k.ls + (k.v * k.sw) * k.ms) + t;
  t -= std::rint(t);
  r.arg = (float)t;
  return r;
}

bool same(float a, float b) { return wgpu::ff::bits(a) == wgpu::ff::bits(b); }

// Returns 1 decided and equal, 0 undecided, -1 decided and different.
int check(const Case &k) {
  const Ref r = reference(k);
  wgpu::ff::Scales cs{split(k.su), split(k.sv), split(k.sw)};
  wgpu::ff::PlanPairs pp{split(k.w0),  split(k.inv_dw),  split(k.c),
                         split(k.ls),  split(k.ms),      k.n_planes > 1,
                         k.ls != 0.0 || k.ms != 0.0};
  float fu, fv, fw, arg;
  if (!wgpu::ff::decide(split(k.u), split(k.v), split(k.w), cs, pp, r.iu0, r.iv0, r.ip, &fu, &fv,
                        &fw, &arg))
    return 0;
  if (same(fu, r.fu) && same(fv, r.fv) && same(fw, r.fw) && same(arg, r.arg)) return 1;
  std::fprintf(stderr, "mismatch: u %.17g su %.17g fu %a/%a fv %a/%a fw %a/%a arg %a/%a\n", k.u,
               k.su, fu, r.fu, fv, r.fv, fw, r.fw, arg, r.arg);
  return -1;
}

// A wide-field-like sample: 20 km baselines, 0.9-1.7 GHz, 3 arcsec pixels on
// a 12288 grid, W = 8, sigma = 1.5.
Case random_case(std::mt19937_64 &g) {
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  Case k;
  const double fl = (0.9e9 + 0.8e9 * uni(g)) / 299792458.0;
  const double gu = 1.4544410433286079e-05 * 12288.0;
  k.su = fl * gu;
  k.sv = fl * gu;
  k.sw = fl;
  const double umax = 6000.0 / k.su;
  k.u = (2.0 * uni(g) - 1.0) * umax;
  k.v = (2.0 * uni(g) - 1.0) * umax;
  k.w = (2.0 * uni(g) - 1.0) * 1500.0;
  k.support = 8;
  const double dw = 1.0 / (1.5 * 0.032);
  const double w_min = -1500.0 * 5.67, w_max = 1500.0 * 5.67;
  k.w0 = w_min - 0.5 * k.support * dw;
  k.inv_dw = 1.0 / dw;
  k.n_planes = (int)std::ceil((w_max - w_min) / dw) + k.support;
  k.c = -0.016 - 0.002 * uni(g);
  // half the samples belong to a shifted image (a facet centre within 3 deg)
  const bool shifted = uni(g) < 0.5;
  k.ls = shifted ? (2.0 * uni(g) - 1.0) * 0.05 : 0.0;
  k.ms = shifted ? (2.0 * uni(g) - 1.0) * 0.05 : 0.0;
  return k;
}

double midpoint_above(float f) {
  return 0.5 * ((double)f + (double)std::nextafter(f, INFINITY));
}

// Cases whose FP64 results lie close to a float rounding boundary (or to a
// half-integer phase), where decide() must either fall back or be right.
Case edge_case(std::mt19937_64 &g, int which) {
  std::uniform_real_distribution<double> uni(0.0, 1.0);
  Case k = random_case(g);
  const double half = 0.5 * k.support;
  // relative offsets log-uniform between 2^-52 and 2^-36: the near ones must
  // fall back, the far ones are decided close to the boundary
  const double jitter = (uni(g) < 0.5 ? -1.0 : 1.0) * std::ldexp(1.0, -52 + (int)(16 * uni(g))) *
                        (1.0 + uni(g));
  if (which == 0) {
    // fu = iu0 - U near the midpoint of two floats in (-W/2, -W/2 + 1]
    const double U = k.u * k.su;
    const int iu0 = (int)std::ceil(U - half);
    const float f = (float)((double)iu0 - U);
    const double target = (double)iu0 - midpoint_above(f) + jitter * std::fabs(U);
    k.u = target / k.su;
  } else if (which == 1 || which == 2) {
    // the phase near a half-integer (1) or its argument near a float
    // midpoint (2): w chosen so that the full phase lands there
    const double tuv = (k.ls != 0.0 || k.ms != 0.0) ? (k.u * k.sw) * k.ls + (k.v * k.sw) * k.ms
                                                     : 0.0;
    const double t = tuv + (k.w * k.sw) * k.c;
    const double n = std::rint(t);
    const double target = which == 1 ? std::floor(t) + 0.5 + jitter * std::fabs(t)
                                     : n + midpoint_above((float)(t - n)) + jitter * std::fabs(t);
    k.w = (target - tuv) / k.c / k.sw;
  } else {
    // fw near a float midpoint
    const double wl = k.w * k.sw;
    const double pw = (wl - k.w0) * k.inv_dw;
    double ip0 = std::ceil(pw - half);
    if (ip0 < 0.0 || ip0 > k.n_planes - k.support) return k;
    const float f = (float)(ip0 - pw);
    const double pw_t = ip0 - midpoint_above(f) + jitter * std::fabs(pw);
    k.w = (pw_t / k.inv_dw + k.w0) / k.sw;
  }
  return k;
}

}  // namespace

int main(int argc, char **argv) {
  const long n_random = argc > 1 ? std::atol(argv[1]) : 1000000;
  const long n_edge = argc > 2 ? std::atol(argv[2]) : 200000;
  const unsigned long seed = argc > 3 ? std::strtoul(argv[3], nullptr, 10) : 1;
  std::mt19937_64 g(seed);
  long dec = 0, bad = 0;
  for (long i = 0; i < n_random; ++i) {
    const int c = check(random_case(g));
    dec += c == 1;
    bad += c < 0;
  }
  std::printf("random %ld decided %ld mismatches %ld\n", n_random, dec, bad);
  long dec_e = 0, bad_e = 0;
  for (long i = 0; i < n_edge; ++i) {
    const int c = check(edge_case(g, (int)(i % 4)));
    dec_e += c == 1;
    bad_e += c < 0;
  }
  std::printf("edge %ld decided %ld mismatches %ld\n", n_edge, dec_e, bad_e);
  return bad + bad_e > 0 ? 1 : 0;
}
