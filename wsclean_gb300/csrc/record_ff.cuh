// Footprint fractions and w phase of a record from float-float arithmetic,
// decided against the FP64 chains they stand for.
//
// The records' fractions are FP64 values rounded to float: fu = fl32(iu0 -
// fl64(u * su)), fv likewise, fw = fl32(ip - fl64(fl64(fl64(w * sw) - w0) *
// inv_dw)), and the phase argument is fl32(t - rint(t)) with
// t = fl64(fl64(w * sw) * c) without shifts, and the same term added to
// fl64(fl64(fl64(u * sw) * l_shift) + fl64(fl64(v * sw) * m_shift)) with them.  Here the same chains run
// on (hi, lo) float pairs (every double split into its nearest float and the
// nearest float to the rest), which carry about 46 significant bits, and each
// result comes with a bound on its distance to the FP64 chain's value.  When
// the float rounding of every candidate is unambiguous under that bound
// (decide() returns true), the floats equal the FP64 chain's results bit for
// bit; otherwise the caller computes the record in FP64.  The functions are
// host and device code so that a CPU test can check the decision against
// FP64 on many inputs (the host build must not contract a * b + c).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define WGPU_FF_HD __host__ __device__ __forceinline__
#else
#define WGPU_FF_HD inline
#endif

namespace wgpu {
namespace ff {

WGPU_FF_HD float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
WGPU_FF_HD float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
WGPU_FF_HD float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
WGPU_FF_HD float ffma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
WGPU_FF_HD int32_t bits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_int(x);
#else
  int32_t b;
  std::memcpy(&b, &x, sizeof(b));
  return b;
#endif
}
WGPU_FF_HD float from_bits(int32_t b) {
#ifdef __CUDA_ARCH__
  return __int_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, sizeof(x));
  return x;
#endif
}

// hi + lo
struct Pair {
  float hi, lo;
};

// A double as its nearest float and the nearest float to the rest (host
// side: tables are split once, not per record).  |x - (hi + lo)| <= 2^-48 |x|.
inline Pair split(double x) {
  const float hi = (float)x;
  return Pair{hi, (float)(x - (double)hi)};
}

// s + e = a + b exactly (Knuth's two-sum).
WGPU_FF_HD Pair two_sum(float a, float b) {
  const float s = fadd(a, b);
  const float bb = fsub(s, a);
  const float e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
  return Pair{s, e};
}

// (a.hi + a.lo)(b.hi + b.lo) within 2^-45 of the exact product of the pairs'
// values, renormalised (|lo| <= ulp(hi)).
WGPU_FF_HD Pair mul(Pair a, Pair b) {
  const float p = fmul(a.hi, b.hi);
  const float e = ffma(a.hi, b.hi, -p);
  const float c = ffma(a.hi, b.lo, ffma(a.lo, b.hi, e));
  const float s = fadd(p, c);
  return Pair{s, fsub(c, fsub(s, p))};
}

// a + b within 2^-47 (|a| + |b|) of the exact sum of the pairs' values
// (renormalised with a full two-sum: the high parts may cancel).
WGPU_FF_HD Pair add(Pair a, Pair b) {
  const Pair d = two_sum(a.hi, b.hi);
  const float c = fadd(d.lo, fadd(a.lo, b.lo));
  return two_sum(d.hi, c);
}

// a - b within 2^-47 (|a| + |b|) of the exact difference of the pairs' values
// (renormalised with a full two-sum: the high parts may cancel).
WGPU_FF_HD Pair sub(Pair a, Pair b) {
  const Pair d = two_sum(a.hi, -b.hi);
  const float c = fadd(d.lo, fsub(a.lo, b.lo));
  return two_sum(d.hi, c);
}

// The half-width of the interval of reals that round to the float t (a quarter
// unit in the last place at a power of two, where the interval is uneven);
// 0 when t is zero, subnormal or not finite (nothing is decided there).
WGPU_FF_HD float half_ulp(float t) {
  const int32_t b = bits(t) & 0x7fffffff;
  const int32_t ex = b & 0x7f800000;
  const int32_t sh = (b & 0x007fffff) == 0 ? 25 : 24;
  if (ex == 0x7f800000 || ex <= (sh << 23)) return 0.0f;
  return from_bits(ex - (sh << 23));
}

// fl32(k - x) for an integer k and the value x of a float pair known to within
// xb of some real X: true (and *out) when fl32(k - X) is the same float for
// every X within that bound.  k - x.hi is formed exactly (two-sum), so the only
// approximations are xb and the rounding of the small remainder.
WGPU_FF_HD bool frac_decided(int k, Pair x, float xb, float *out) {
  const Pair d = two_sum((float)k, -x.hi);  // k is an exact float (|k| < 2^24)
  const float r = fsub(d.lo, x.lo);
  const float rb = fmul(fabsf(r), 1.2e-7f);  // rounding of r (2^-23 |r|)
  const Pair t = two_sum(d.hi, r);
  const float hu = half_ulp(t.hi);
  if (!(fabsf(t.lo) + xb + rb < hu)) return false;
  *out = t.hi;
  return true;
}

// Constants of one plan and channel, split into pairs.
struct Scales {
  Pair su, sv, sw;  // per channel
};
struct PlanPairs {
  Pair w0, inv_dw, c;  // w0, 1 / dw, c_n (the n - 1 centre)
  Pair l, m;           // l_shift, m_shift
  bool w_planes;       // n_planes > 1
  bool shift;          // the phase has the l and m terms
};

// 2^-43: the bound factor of every chain below.  A float-float product is
// within 2^-45.5 of the exact product of its operands' values (two roundings
// of the cross terms and the dropped lo * lo term), a difference within 2^-47,
// each FP64 step rounds at 2^-53 and the splits of the inputs are within
// 2^-48.  The longest chain (the phase: two products after the splits) stays
// within 2^-44.1 of the FP64 value, relative to the magnitudes the bounds
// below name; 2^-43 leaves a factor two.
constexpr float kBound = 1.1368683772161603e-13f;  // 2^-43

// Fractions and phase argument of a record with integer corner (iu0, iv0, ip)
// already decided; u, v, w the row's coordinates as pairs.  True when fu, fv,
// fw and arg equal the FP64 chains' results (see the file comment).
WGPU_FF_HD bool decide(Pair u, Pair v, Pair w, const Scales &cs, const PlanPairs &pp, int iu0,
                       int iv0, int ip, float *fu, float *fv, float *fw, float *arg) {
  const Pair U = mul(u, cs.su);
  if (!frac_decided(iu0, U, fmul(kBound, fabsf(U.hi)), fu)) return false;
  const Pair V = mul(v, cs.sv);
  if (!frac_decided(iv0, V, fmul(kBound, fabsf(V.hi)), fv)) return false;
  const Pair wl = mul(w, cs.sw);
  if (pp.w_planes) {
    const Pair d = sub(wl, pp.w0);
    const Pair pw = mul(d, pp.inv_dw);
    const float b = fmul(kBound, fadd(fmul(fabsf(pp.inv_dw.hi),
                                           fadd(fadd(fabsf(wl.hi), fabsf(pp.w0.hi)),
                                                fabsf(d.hi))),
                                      fabsf(pw.hi)));
    if (!frac_decided(ip, pw, b, fw)) return false;
  } else {
    *fw = 0.0f;
  }
  // phase: t = fl64(wl c) without shifts; with them
  // t = fl64(fl64(fl64(fl64(u f) l) + fl64(fl64(v f) m)) + fl64(wl c)), f the
  // channel's w scale (the chain the FP64 record pass rounds step by step);
  // then reduced by its nearest integer
  Pair t = mul(wl, pp.c);
  float tb = fmul(kBound, fabsf(t.hi));
  if (pp.shift) {
    const Pair tu = mul(mul(u, cs.sw), pp.l), tv = mul(mul(v, cs.sw), pp.m);
    const Pair t12 = add(tu, tv);
    const Pair t3 = t;
    t = add(t12, t3);
    // each term's product chain, the two sums and their FP64 roundings,
    // relative to the magnitudes involved
    tb = fmul(kBound, fadd(fadd(fadd(fabsf(tu.hi), fabsf(tv.hi)), fadd(fabsf(t3.hi),
                                                                      fabsf(t12.hi))),
                           fabsf(t.hi)));
  }
  if (!(fabsf(t.hi) < 4194304.0f)) return false;  // 2^22
  const float n = rintf(t.hi);
  const Pair f = two_sum(fsub(t.hi, n), t.lo);  // t.hi - n is exact
  if (!(fabsf(f.hi) + fabsf(f.lo) + tb < 0.4999f)) return false;  // rint(t) == n
  const float hu = half_ulp(f.hi);
  if (!(fabsf(f.lo) + tb < hu)) return false;
  *arg = f.hi;
  return true;
}

}  // namespace ff
}  // namespace wgpu
