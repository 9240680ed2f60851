// Complex float2 helpers and the conversions between one Stokes (or single
// correlation) value and the four linear correlations (XX, XY, YX, YY), shared
// by the gain kernels and the raw-row preparation.
#pragma once

#include <cuda_runtime.h>

namespace wgpu {

__device__ __forceinline__ float2 cm(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 ca(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cs(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// One value from the four linear correlations: Stokes I, Q, U, V (pol 0-3,
// standard linear-feed conversion with a factor 1/2) or one correlation
// (pol 4-7), as CollapseData<4> does (gridding/msgridderdata.h:46-50).
__device__ __forceinline__ float2 collapse4(const float2 *v, int pol) {
  switch (pol) {
    case 0: return cs(ca(v[0], v[3]), 0.5f);
    case 1: return make_float2(0.5f * (v[0].x - v[3].x), 0.5f * (v[0].y - v[3].y));
    case 2: return cs(ca(v[1], v[2]), 0.5f);
    case 3: {
      const float2 d = make_float2(v[2].x - v[1].x, v[2].y - v[1].y);
      return make_float2(-0.5f * d.y, 0.5f * d.x);
    }
    case 4: return v[0];
    case 5: return v[1];
    case 6: return v[2];
    default: return v[3];
  }
}

// Stokes parameter `pol` (or linear correlation 4-7) of value s as linear
// correlations (XX, XY, YX, YY): XX = I + Q, YY = I - Q, XY = U + iV,
// YX = U - iV, the inverse of collapse4 (4-polarisation ExpandData,
// msgridderdata.h:63-68).
__device__ __forceinline__ void expand4(float2 s, int pol, float2 *v) {
  const float2 z = make_float2(0.f, 0.f);
  v[0] = v[1] = v[2] = v[3] = z;
  switch (pol) {
    case 0: v[0] = s; v[3] = s; break;
    case 1: v[0] = s; v[3] = make_float2(-s.x, -s.y); break;
    case 2: v[1] = s; v[2] = s; break;
    case 3: v[1] = make_float2(-s.y, s.x); v[2] = make_float2(s.y, -s.x); break;
    case 4: v[0] = s; break;
    case 5: v[1] = s; break;
    case 6: v[2] = s; break;
    default: v[3] = s; break;
  }
}

// r = a^H b (row-major 2x2)
__device__ __forceinline__ void herm_mul(const float2 *a, const float2 *b, float2 *r) {
  const float2 h[4] = {cj(a[0]), cj(a[2]), cj(a[1]), cj(a[3])};
  r[0] = ca(cm(h[0], b[0]), cm(h[1], b[2]));
  r[1] = ca(cm(h[0], b[1]), cm(h[1], b[3]));
  r[2] = ca(cm(h[2], b[0]), cm(h[3], b[2]));
  r[3] = ca(cm(h[2], b[1]), cm(h[3], b[3]));
}
__device__ __forceinline__ void mat_mul(const float2 *a, const float2 *b, float2 *r) {
  r[0] = ca(cm(a[0], b[0]), cm(a[1], b[2]));
  r[1] = ca(cm(a[0], b[1]), cm(a[1], b[3]));
  r[2] = ca(cm(a[2], b[0]), cm(a[3], b[2]));
  r[3] = ca(cm(a[2], b[1]), cm(a[3], b[3]));
}

// ApplyConjugatedGain (visibilitymodifier.h:378-401) on the NPOL correlations
// of one sample, before weighting and collapse: XX and YY (one correlation)
// conj(g1) V g2 with the matching diagonal element, TRACE V times half the
// sum of g2[k] conj(g1[k]), 2VIS_DIAGONAL the diagonal pair with the second
// term using the updated first (visibilitymodifier.h:393-396), FULL
// G1^H V G2.
template <int NPOL>
__device__ __forceinline__ void apply_conjugated_gain(int mode, float2 *v, const float2 *g1,
                                                      const float2 *g2) {
  if constexpr (NPOL == 1) {
    if (mode == 0) {
      v[0] = cm(cm(cj(g1[0]), v[0]), g2[0]);
    } else if (mode == 1) {
      v[0] = cm(cm(cj(g1[3]), v[0]), g2[3]);
    } else {
      float2 dd = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < 4; ++k) dd = ca(dd, cm(g2[k], cj(g1[k])));
      v[0] = cm(v[0], cs(dd, 0.5f));
    }
  } else if constexpr (NPOL == 2) {
    const float2 v0 = ca(cm(cm(cj(g1[0]), v[0]), g2[0]), cm(cm(cj(g1[2]), v[1]), g2[2]));
    const float2 v1 = ca(cm(cm(cj(g1[3]), v[1]), g2[3]), cm(cm(cj(g1[1]), v0), g2[1]));
    v[0] = v0;
    v[1] = v1;
  } else {
    float2 t1[4];
    herm_mul(g1, v, t1);
    mat_mul(t1, g2, v);
  }
}

}  // namespace wgpu
