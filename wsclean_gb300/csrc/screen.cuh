// Fixed-point w-screen phase terms, shared by the per-plan table kernel
// (correct.cu), the column passes (fft.cu) and a host test.
//
// The screen of plane q at a pixel with n - 1 - c_n = nu is exp(-+2 pi i t),
// t = (w0 + q dw) nu turns.  The FP64 products w0 nu and dw nu are reduced
// modulo one turn once per plan and pixel and kept as 32-bit fixed-point turns
// a and k (rounded to 2^-33 turns), with r = the part of dw nu below 2^-33.
// For plane q, a + q k in wrapping uint32 arithmetic is (w0 + q dw) nu modulo
// one turn for every q; converting it to float and adding q r costs two FP32
// roundings, about 5e-8 turns, less than rounding the reduced FP64 argument
// to FP32.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define WGPU_SCREEN_HD __host__ __device__ __forceinline__
#else
#define WGPU_SCREEN_HD inline
#endif

namespace wgpu {

struct ScreenTerms {
  uint32_t a, k;
  float r;
};

// The terms of one pixel (FP64, once per plan).
WGPU_SCREEN_HD ScreenTerms screen_terms(double w0, double dw, double nu) {
  constexpr double kTurn = 4294967296.0;  // 2^32
  double a = w0 * nu;
  a -= rint(a);
  double k = dw * nu;
  k -= rint(k);
  const double kq = rint(k * kTurn);
  ScreenTerms t;
  t.a = (uint32_t)(int64_t)rint(a * kTurn);
  t.k = (uint32_t)(int64_t)kq;
  t.r = (float)(k - kq * (1.0 / kTurn));
  return t;
}

// 2 t of plane q in FP32, within about [-1, 1]: sincospi of it gives the
// screen's cosine and sine.
WGPU_SCREEN_HD float screen_arg2(uint32_t a, uint32_t k, float r, int q) {
  const int32_t t = (int32_t)(a + (uint32_t)q * k);  // turns in 2^-32, in [-1/2, 1/2)
  return fmaf((float)t, 0x1p-31f, (float)(2 * q) * r);
}

}  // namespace wgpu
