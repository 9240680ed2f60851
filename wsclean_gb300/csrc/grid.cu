// K2 gridding and K3 degridding over (uv tile, w-plane group) work units.
//
// Gridding: one CTA owns a T x T tile of G consecutive w planes.  It reads the
// visibilities bucketed in its own tile and in the three neighbouring tiles
// whose footprints can spill into it (left, below, below-left; the footprint
// corner decides the bucket), restricted by key range to the first planes that
// reach the group.  A chunk of records at a time is spread into a shared-
// memory copy of the tile with shared-memory atomics; after each chunk the
// partial tile is folded into per-thread Kahan-compensated accumulators and
// cleared, so long buckets do not lose FP32 precision.  Each tile cell is
// finally written once to HBM (no global atomics, no memset of the planes).
//
// Degridding: one CTA loads its tile plus a (W-1)-cell halo of G planes into
// shared memory and gathers, for every visibility of its own bucket, the
// W x W x (planes in the group) weighted sum; results are added to the
// per-visibility accumulator.
#include "wgpu_internal.h"

namespace wgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 64;  // records staged per round
constexpr int kCells = 4096;  // G * T * T cells per gridding CTA
constexpr int kCellsPerThread = kCells / kThreads;

__device__ __forceinline__ float es_eval(float beta, float z) {
  const float t = 1.0f - z * z;
  return t > 0.0f ? expf(beta * (sqrtf(t) - 1.0f)) : 0.0f;
}

__device__ __forceinline__ VisRecord load_record(const VisRecord *r) {
  const float4 a = __ldg(reinterpret_cast<const float4 *>(r));
  const float4 b = __ldg(reinterpret_cast<const float4 *>(r) + 1);
  VisRecord o;
  o.re = a.x;
  o.im = a.y;
  o.fu = a.z;
  o.fv = a.w;
  o.fw = b.x;
  o.iu = __float_as_int(b.y);
  o.iv = __float_as_int(b.z);
  o.ip = __float_as_int(b.w);
  return o;
}

template <int T, int G>
__global__ void __launch_bounds__(kThreads)
    grid_kernel(DevPlan p, const VisRecord *__restrict__ rec,
                const uint32_t *__restrict__ off, int p_begin, int n_batch,
                float2 *__restrict__ planes) {
  static_assert(G * T * T == kCells, "cells per CTA");
  constexpr int TS = T + 1;  // padded row stride (float2 units)
  __shared__ float2 buf[G * T * TS];
  __shared__ float kval[kChunk][3][kMaxSupport];
  __shared__ float2 cvis[kChunk];
  __shared__ int cpos[kChunk][3];  // iu_rel, iv_rel, ip
  __shared__ float cfrac[kChunk][3];  // fu, fv, fw

  const int W = p.support;
  const float inv_half = 2.0f / (float)W;
  const int tile = blockIdx.x;
  const int tu = tile % p.ntu, tv = tile / p.ntu;
  const int q0 = p_begin + blockIdx.y * G;
  const int q1 = min(q0 + G, p_begin + n_batch);

  for (int c = threadIdx.x; c < G * T * TS; c += kThreads) buf[c] = make_float2(0.f, 0.f);
  float2 sum[kCellsPerThread], comp[kCellsPerThread];
#pragma unroll
  for (int k = 0; k < kCellsPerThread; ++k) {
    sum[k] = make_float2(0.f, 0.f);
    comp[k] = make_float2(0.f, 0.f);
  }
  __syncthreads();

  const int plo = max(q0 - W + 1, 0);
  const int phi = min(q1 - 1, p.n_planes - 1);
  for (int nb = 0; nb < 4; ++nb) {
    const int dtu = nb & 1, dtv = nb >> 1;
    const int stu = (tu - dtu + p.ntu) % p.ntu;
    const int stv = (tv - dtv + p.ntv) % p.ntv;
    const uint32_t key0 = (uint32_t)(stv * p.ntu + stu) * (uint32_t)p.n_planes;
    const uint32_t s0 = off[key0 + plo];
    const uint32_t s1 = off[key0 + phi + 1];
    for (uint32_t sb = s0; sb < s1; sb += kChunk) {
      const int m_count = (int)min((uint32_t)kChunk, s1 - sb);
      if (threadIdx.x < m_count) {
        const VisRecord r = load_record(rec + sb + threadIdx.x);
        int iu_rel = r.iu - tu * T;
        if (iu_rel >= T) iu_rel -= p.nu;
        int iv_rel = r.iv - tv * T;
        if (iv_rel >= T) iv_rel -= p.nv;
        cvis[threadIdx.x] = make_float2(r.re, r.im);
        cpos[threadIdx.x][0] = iu_rel;
        cpos[threadIdx.x][1] = iv_rel;
        cpos[threadIdx.x][2] = r.ip;
        cfrac[threadIdx.x][0] = r.fu;
        cfrac[threadIdx.x][1] = r.fv;
        cfrac[threadIdx.x][2] = r.fw;
      }
      __syncthreads();
      // kernel values: (m, dim, j) -> phi((f + j) / half)
      for (int idx = threadIdx.x; idx < m_count * 3 * kMaxSupport; idx += kThreads) {
        const int j = idx % kMaxSupport;
        const int d = (idx / kMaxSupport) % 3;
        const int m = idx / (3 * kMaxSupport);
        if (j >= W) continue;
        float v;
        if (d == 2 && p.n_planes == 1)
          v = (j == 0) ? 1.0f : 0.0f;
        else
          v = es_eval(p.beta, (cfrac[m][d] + (float)j) * inv_half);
        kval[m][d][j] = v;
      }
      __syncthreads();
      // spread: units (m, j) = one footprint row of one visibility
      for (int u = threadIdx.x; u < m_count * W; u += kThreads) {
        const int m = u / W, j = u - m * W;
        const int row = cpos[m][1] + j;
        if (row < 0 || row >= T) continue;
        const int ip = cpos[m][2];
        const int pa = max(ip, q0), pb = min(ip + W - 1, q1 - 1);
        if (pa > pb) continue;
        const int iu_rel = cpos[m][0];
        const int ia = max(0, -iu_rel), ib = min(W - 1, T - 1 - iu_rel);
        const float ky = kval[m][1][j];
        const float2 v = cvis[m];
        for (int q = pa; q <= pb; ++q) {
          const float wy = ky * kval[m][2][q - ip];
          float2 *brow = buf + ((q - q0) * T + row) * TS + iu_rel;
          for (int i = ia; i <= ib; ++i) {
            const float wt = wy * kval[m][0][i];
            atomicAdd(&brow[i].x, wt * v.x);
            atomicAdd(&brow[i].y, wt * v.y);
          }
        }
      }
      __syncthreads();
      // fold the chunk into the compensated accumulators
#pragma unroll
      for (int k = 0; k < kCellsPerThread; ++k) {
        const int c = threadIdx.x + k * kThreads;
        const int pq = c / (T * T), rem = c - pq * T * T;
        const int row = rem / T, col = rem - row * T;
        float2 *cell = buf + (pq * T + row) * TS + col;
        const float2 x = *cell;
        *cell = make_float2(0.f, 0.f);
        // Kahan (Neumaier form) per component
        float y = x.x - comp[k].x;
        float t = sum[k].x + y;
        comp[k].x = (t - sum[k].x) - y;
        sum[k].x = t;
        y = x.y - comp[k].y;
        t = sum[k].y + y;
        comp[k].y = (t - sum[k].y) - y;
        sum[k].y = t;
      }
      __syncthreads();
    }
  }
  // write the tile of each plane in the group
  const size_t plane_elems = (size_t)p.nu * p.nv;
#pragma unroll
  for (int k = 0; k < kCellsPerThread; ++k) {
    const int c = threadIdx.x + k * kThreads;
    const int pq = c / (T * T), rem = c - pq * T * T;
    const int row = rem / T, col = rem - row * T;
    const int q = q0 + pq;
    if (q < q1) {
      planes[(size_t)(q - p_begin) * plane_elems + (size_t)(tv * T + row) * p.nu +
             tu * T + col] = sum[k];
    }
  }
}

template <int T, int G>
__global__ void __launch_bounds__(kThreads)
    degrid_kernel(DevPlan p, const VisRecord *__restrict__ rec,
                  const uint32_t *__restrict__ off, int p_begin, int n_batch,
                  const float2 *__restrict__ planes, float2 *__restrict__ acc) {
  extern __shared__ float2 region[];  // [G][R][RS]
  const int W = p.support;
  const int R = T + W - 1;
  const int RS = R + 1;
  const float half = 0.5f * (float)W;
  const float inv_half = 1.0f / half;
  const int tile = blockIdx.x;
  const int tu = tile % p.ntu, tv = tile / p.ntu;
  const int q0 = p_begin + blockIdx.y * G;
  const int q1 = min(q0 + G, p_begin + n_batch);
  const int plo = max(q0 - W + 1, 0);
  const int phi = min(q1 - 1, p.n_planes - 1);
  const uint32_t key0 = (uint32_t)tile * (uint32_t)p.n_planes;
  const uint32_t s0 = off[key0 + plo];
  const uint32_t s1 = off[key0 + phi + 1];
  if (s0 == s1) return;  // uniform across the CTA

  const size_t plane_elems = (size_t)p.nu * p.nv;
  const int nq = q1 - q0;
  for (int idx = threadIdx.x; idx < nq * R * R; idx += blockDim.x) {
    const int pq = idx / (R * R), rem = idx - pq * R * R;
    const int r = rem / R, c = rem - r * R;
    int gv = tv * T + r;
    if (gv >= p.nv) gv -= p.nv;
    int gu = tu * T + c;
    if (gu >= p.nu) gu -= p.nu;
    region[(pq * R + r) * RS + c] =
        planes[(size_t)(q0 + pq - p_begin) * plane_elems + (size_t)gv * p.nu + gu];
  }
  __syncthreads();

  for (uint32_t s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
    const VisRecord r = load_record(rec + s);
    float kx[kMaxSupport], ky[kMaxSupport];
#pragma unroll
    for (int j = 0; j < kMaxSupport; ++j) {
      kx[j] = j < W ? es_eval(p.beta, (r.fu + (float)j) * inv_half) : 0.0f;
      ky[j] = j < W ? es_eval(p.beta, (r.fv + (float)j) * inv_half) : 0.0f;
    }
    const int iu_rel = r.iu - tu * T;
    const int iv_rel = r.iv - tv * T;
    const int pa = max(r.ip, q0), pb = min(r.ip + W - 1, q1 - 1);
    float sr = 0.f, si = 0.f;
    for (int q = pa; q <= pb; ++q) {
      const float kw = p.n_planes == 1 ? 1.0f
                                       : es_eval(p.beta, (r.fw + (float)(q - r.ip)) * inv_half);
      const float2 *base = region + ((q - q0) * R + iv_rel) * RS + iu_rel;
      float pr = 0.f, pi = 0.f;
      for (int j = 0; j < W; ++j) {
        const float2 *rowp = base + j * RS;
        float rr = 0.f, ri = 0.f;
#pragma unroll
        for (int i = 0; i < kMaxSupport; ++i) {
          if (i < W) {
            const float2 g = rowp[i];
            rr += kx[i] * g.x;
            ri += kx[i] * g.y;
          }
        }
        pr += ky[j] * rr;
        pi += ky[j] * ri;
      }
      sr += kw * pr;
      si += kw * pi;
    }
    atomicAdd(&acc[s], make_float2(sr, si));
  }
}

}  // namespace

int grid_plane_group() { return 4; }

void launch_grid(const DevPlan &p, const VisRecord *rec, const uint32_t *off,
                 int p_begin, int n_batch, float2 *planes, cudaStream_t s) {
  const int n_tiles = p.ntu * p.ntv;
  if (p.tile == 32) {
    constexpr int G = 4;
    dim3 grid(n_tiles, (n_batch + G - 1) / G);
    grid_kernel<32, G><<<grid, kThreads, 0, s>>>(p, rec, off, p_begin, n_batch, planes);
  } else if (p.tile == 16) {
    constexpr int G = 16;
    dim3 grid(n_tiles, (n_batch + G - 1) / G);
    grid_kernel<16, G><<<grid, kThreads, 0, s>>>(p, rec, off, p_begin, n_batch, planes);
  } else {
    throw Error(WGPU_ERR_INVALID, "tile must be 16 or 32");
  }
  check_launch("grid_kernel");
}

void launch_degrid(const DevPlan &p, const VisRecord *rec, const uint32_t *off,
                   int p_begin, int n_batch, const float2 *planes, float2 *acc,
                   cudaStream_t s) {
  const int n_tiles = p.ntu * p.ntv;
  const int R = p.tile + p.support - 1;
  if (p.tile == 32) {
    constexpr int G = 4;
    const size_t smem = sizeof(float2) * G * R * (R + 1);
    cudaFuncSetAttribute(degrid_kernel<32, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(n_tiles, (n_batch + G - 1) / G);
    degrid_kernel<32, G><<<grid, kThreads, smem, s>>>(p, rec, off, p_begin, n_batch, planes, acc);
  } else if (p.tile == 16) {
    constexpr int G = 8;
    const size_t smem = sizeof(float2) * G * R * (R + 1);
    cudaFuncSetAttribute(degrid_kernel<16, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(n_tiles, (n_batch + G - 1) / G);
    degrid_kernel<16, G><<<grid, kThreads, smem, s>>>(p, rec, off, p_begin, n_batch, planes, acc);
  } else {
    throw Error(WGPU_ERR_INVALID, "tile must be 16 or 32");
  }
  check_launch("degrid_kernel");
}

}  // namespace wgpu
