// K2 gridding and K3 degridding over (uv tile, w-plane group) work units.
//
// Work unit = (uv tile T x T, group of G consecutive w planes).  A gridding
// unit reads the visibilities bucketed in its own tile and in the three
// neighbouring tiles whose footprints can spill into it (left, below,
// below-left; the footprint corner decides the bucket), restricted by key
// range to the first planes that reach the group.  Units are split into work
// items of at most kItemVis visibility reads, and one persistent launch works
// through the items of a plane batch from a device counter, so that the
// crowded tiles of a dense uv core are shared by many CTAs.
//
// Gridding item: records are staged kChunk at a time in shared memory and
// spread into a shared copy of the tile with shared-memory atomics; every
// kFoldEvery rounds the partial tile is folded into per-thread
// Kahan-compensated accumulators and cleared, so long lists keep FP32
// precision.  A unit made of one item writes each cell once to HBM; the items
// of a split unit add into cells that a planning pass zeroed.
//
// Degridding item: loads its tile plus a (W-1)-cell halo of G planes into
// shared memory and gathers, for each visibility of its slice of the own
// bucket, the W x W x (planes in the group) weighted sum, added to the
// per-visibility accumulator.
#include "wgpu_internal.h"

namespace wgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 64;       // records staged in shared memory per round
constexpr int kFoldEvery = 4;    // rounds between two Kahan folds
constexpr uint32_t kItemVis = 2048;  // visibility reads per work item

// ES kernel phi(z) = exp(beta (sqrt(1 - z^2) - 1)), 0 outside |z| < 1, with the
// fast intrinsics: their relative error (~1e-7 where phi is large) is white
// noise well inside the FP32 budget the planner accounts for.
__device__ __forceinline__ float es_eval(float beta, float z) {
  const float t = 1.0f - z * z;
  return t > 0.0f ? __expf(beta * (t * rsqrtf(t) - 1.0f)) : 0.0f;
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

// Key layout (bucket.cu): key = ((tile * 4 + class) * n_planes + first plane),
// class = which neighbours a footprint spills into (0 none, 1 right, 2 right
// and up, 3 up).  A gridding unit reads its own tile (all classes), the left
// tile (classes 1-2), the lower tile (2-3) and the lower-left tile (2): nine
// key ranges, each restricted to first planes that reach the plane group.
__constant__ int kRangeDtu[9] = {0, 0, 0, 0, 1, 1, 0, 0, 1};
__constant__ int kRangeDtv[9] = {0, 0, 0, 0, 0, 0, 1, 1, 1};
__constant__ int kRangeCls[9] = {0, 1, 2, 3, 1, 2, 2, 3, 2};

__device__ __forceinline__ void unit_range(const DevPlan &p, const uint32_t *off, int tile,
                                           int q0, int q1, int r, uint32_t *s0,
                                           uint32_t *s1) {
  const int tu = tile % p.ntu, tv = tile / p.ntu;
  const int stu = (tu - kRangeDtu[r] + p.ntu) % p.ntu;
  const int stv = (tv - kRangeDtv[r] + p.ntv) % p.ntv;
  const int plo = max(q0 - p.support + 1, 0);
  const int phi = min(q1 - 1, p.n_planes - 1);
  const uint32_t key0 =
      ((uint32_t)(stv * p.ntu + stu) * 4u + (uint32_t)kRangeCls[r]) * (uint32_t)p.n_planes;
  *s0 = __ldg(off + key0 + plo);
  *s1 = __ldg(off + key0 + phi + 1);
}

// Planning pass: one warp per unit counts the unit's visibility reads and its
// work items; the cells of split gridding units are zeroed here.
template <int T, int G>
__global__ void __launch_bounds__(kThreads)
    grid_plan_kernel(DevPlan p, const uint32_t *__restrict__ off, int p_begin, int n_batch,
                     int n_units, int degrid, uint32_t *__restrict__ items,
                     uint32_t *__restrict__ counts, float2 *__restrict__ planes) {
  const int unit = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (unit >= n_units) return;
  const int n_tiles = p.ntu * p.ntv;
  const int tile = unit % n_tiles, group = unit / n_tiles;
  const int q0 = p_begin + group * G;
  const int q1 = min(q0 + G, p_begin + n_batch);
  uint32_t cnt = 0;
  if (lane < (degrid ? 4 : 9)) {
    uint32_t a, b;
    unit_range(p, off, tile, q0, q1, lane, &a, &b);
    cnt = b - a;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  uint32_t n_items = (cnt + kItemVis - 1) / kItemVis;
  if (!degrid && n_items == 0) n_items = 1;  // an empty tile still writes zeros
  if (lane == 0) {
    items[unit] = n_items;
    counts[unit] = cnt;
  }
  if (!degrid && n_items > 1) {
    const int tu = tile % p.ntu, tv = tile / p.ntu;
    const size_t plane_elems = (size_t)p.nu * p.nv;
    for (int c = lane; c < (q1 - q0) * T * T; c += 32) {
      const int pq = c / (T * T), rem = c - pq * T * T;
      const int row = rem / T, col = rem - row * T;
      planes[(size_t)(q0 + pq - p_begin) * plane_elems + (size_t)(tv * T + row) * p.nu +
             tu * T + col] = make_float2(0.f, 0.f);
    }
  }
}

// item -> unit descriptors (bit 31 marks a unit without visibilities).
__global__ void fill_items_kernel(const uint32_t *__restrict__ item_off,
                                  const uint32_t *__restrict__ counts, int n_units,
                                  uint32_t *__restrict__ desc) {
  const int unit = blockIdx.x * blockDim.x + threadIdx.x;
  if (unit >= n_units) return;
  const uint32_t a = item_off[unit], b = item_off[unit + 1];
  const uint32_t flag = counts[unit] == 0 ? 0x80000000u : 0u;
  for (uint32_t i = a; i < b; ++i) desc[i] = (uint32_t)unit | flag;
}

template <int T, int G>
__global__ void __launch_bounds__(kThreads)
    grid_kernel(DevPlan p, const VisRecord *__restrict__ rec,
                const uint32_t *__restrict__ off, int p_begin, int n_batch,
                const uint32_t *__restrict__ item_off, const uint32_t *__restrict__ desc,
                uint32_t total, float2 *__restrict__ planes) {
  constexpr int kCellsPerThread = G * T * T / kThreads;  // cells a thread folds
  static_assert(kCellsPerThread * kThreads == G * T * T, "cells per work item");
  constexpr int TS = T + 1;  // padded row stride (float2 units)
  __shared__ float2 buf[G * T * TS];
  __shared__ float kval[kChunk][3][kMaxSupport];
  __shared__ float2 cvis[kChunk];
  __shared__ int cpos[kChunk][3];     // iu_rel, iv_rel, ip
  __shared__ float cfrac[kChunk][3];  // fu, fv, fw

  const int W = p.support;
  const float inv_half = 2.0f / (float)W;
  const int n_tiles = p.ntu * p.ntv;
  const size_t plane_elems = (size_t)p.nu * p.nv;

  for (int c = threadIdx.x; c < G * T * TS; c += kThreads) buf[c] = make_float2(0.f, 0.f);
  __syncthreads();

  // static round-robin over the work items: no shared fetch, no barrier
  for (uint32_t item = blockIdx.x; item < total; item += gridDim.x) {
    const uint32_t d = __ldg(desc + item);
    const int unit = (int)(d & 0x7fffffffu);
    const int tile = unit % n_tiles, group = unit / n_tiles;
    const int tu = tile % p.ntu, tv = tile / p.ntu;
    const int q0 = p_begin + group * G;
    const int q1 = min(q0 + G, p_begin + n_batch);
    if (d & 0x80000000u) {
      // no visibility reaches this unit: its cells are zero
      for (int c = threadIdx.x; c < (q1 - q0) * T * T; c += kThreads) {
        const int pq = c / (T * T), rem = c - pq * T * T;
        const int row = rem / T, col = rem - row * T;
        planes[(size_t)(q0 + pq - p_begin) * plane_elems + (size_t)(tv * T + row) * p.nu +
               tu * T + col] = make_float2(0.f, 0.f);
      }
      continue;
    }
    const uint32_t first = __ldg(item_off + unit);
    const uint32_t n_items = __ldg(item_off + unit + 1) - first;
    const uint32_t lo = (item - first) * kItemVis, hi = lo + kItemVis;

    float2 sum[kCellsPerThread], comp[kCellsPerThread];
#pragma unroll
    for (int k = 0; k < kCellsPerThread; ++k) {
      sum[k] = make_float2(0.f, 0.f);
      comp[k] = make_float2(0.f, 0.f);
    }
    int rounds = 0;
    uint32_t base = 0;  // position of range r in the unit's concatenated list
    for (int r = 0; r < 9; ++r) {
      uint32_t s0, s1;
      unit_range(p, off, tile, q0, q1, r, &s0, &s1);
      const uint32_t len = s1 - s0;
      const uint32_t a = max(lo, base), b = min(hi, base + len);
      const uint32_t start = base;
      base += len;
      if (a >= b) continue;
      const uint32_t e0 = s0 + (a - start), e1 = s0 + (b - start);
      for (uint32_t sb = e0; sb < e1; sb += kChunk) {
        const int m_count = (int)min((uint32_t)kChunk, e1 - sb);
        if (threadIdx.x < m_count) {
          const VisRecord rr = load_record(rec + sb + threadIdx.x);
          int iu_rel = rr.iu - tu * T;
          if (iu_rel >= T) iu_rel -= p.nu;
          int iv_rel = rr.iv - tv * T;
          if (iv_rel >= T) iv_rel -= p.nv;
          cvis[threadIdx.x] = make_float2(rr.re, rr.im);
          cpos[threadIdx.x][0] = iu_rel;
          cpos[threadIdx.x][1] = iv_rel;
          cpos[threadIdx.x][2] = rr.ip;
          cfrac[threadIdx.x][0] = rr.fu;
          cfrac[threadIdx.x][1] = rr.fv;
          cfrac[threadIdx.x][2] = rr.fw;
        }
        __syncthreads();
        // kernel values: (m, dim, j) -> phi((f + j) / half)
        for (int idx = threadIdx.x; idx < m_count * 3 * kMaxSupport; idx += kThreads) {
          const int j = idx % kMaxSupport;
          const int dd = (idx / kMaxSupport) % 3;
          const int m = idx / (3 * kMaxSupport);
          if (j >= W) continue;
          float v;
          if (dd == 2 && p.n_planes == 1)
            v = (j == 0) ? 1.0f : 0.0f;
          else
            v = es_eval(p.beta, (cfrac[m][dd] + (float)j) * inv_half);
          kval[m][dd][j] = v;
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
        if (++rounds == kFoldEvery) {
          rounds = 0;
#pragma unroll
          for (int k = 0; k < kCellsPerThread; ++k) {
            const int c = threadIdx.x + k * kThreads;
            const int pq = c / (T * T), rem = c - pq * T * T;
            const int row = rem / T, col = rem - row * T;
            float2 *cell = buf + (pq * T + row) * TS + col;
            const float2 x = *cell;
            *cell = make_float2(0.f, 0.f);
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
    }
    // final fold and write
#pragma unroll
    for (int k = 0; k < kCellsPerThread; ++k) {
      const int c = threadIdx.x + k * kThreads;
      const int pq = c / (T * T), rem = c - pq * T * T;
      const int row = rem / T, col = rem - row * T;
      float2 *cell = buf + (pq * T + row) * TS + col;
      const float2 x = *cell;
      *cell = make_float2(0.f, 0.f);
      float y = x.x - comp[k].x;
      float t = sum[k].x + y;
      comp[k].x = (t - sum[k].x) - y;
      sum[k].x = t;
      y = x.y - comp[k].y;
      t = sum[k].y + y;
      comp[k].y = (t - sum[k].y) - y;
      sum[k].y = t;
      const int q = q0 + pq;
      if (q < q1) {
        float2 *dst = planes + (size_t)(q - p_begin) * plane_elems +
                      (size_t)(tv * T + row) * p.nu + tu * T + col;
        if (n_items == 1)
          *dst = sum[k];
        else
          atomicAdd(dst, sum[k]);
      }
    }
    __syncthreads();
  }
}

template <int T, int G>
__global__ void __launch_bounds__(kThreads)
    degrid_kernel(DevPlan p, const VisRecord *__restrict__ rec,
                  const uint32_t *__restrict__ off, int p_begin, int n_batch,
                  const uint32_t *__restrict__ item_off, const uint32_t *__restrict__ desc,
                  uint32_t total, const float2 *__restrict__ planes,
                  float2 *__restrict__ acc) {
  extern __shared__ float2 region[];  // [G][R][RS]
  const int W = p.support;
  const int R = T + W - 1;
  const int RS = R + 1;
  const float inv_half = 2.0f / (float)W;
  const int n_tiles = p.ntu * p.ntv;
  const size_t plane_elems = (size_t)p.nu * p.nv;

  for (uint32_t item = blockIdx.x; item < total; item += gridDim.x) {
    const int unit = (int)(__ldg(desc + item) & 0x7fffffffu);
    const int tile = unit % n_tiles, group = unit / n_tiles;
    const int tu = tile % p.ntu, tv = tile / p.ntu;
    const int q0 = p_begin + group * G;
    const int q1 = min(q0 + G, p_begin + n_batch);
    const uint32_t lo = (item - __ldg(item_off + unit)) * kItemVis, hi = lo + kItemVis;

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

    uint32_t base = 0;
    for (int rg = 0; rg < 4; ++rg) {  // own tile, classes 0..3
      uint32_t s0, s1;
      unit_range(p, off, tile, q0, q1, rg, &s0, &s1);
      const uint32_t len = s1 - s0;
      const uint32_t a = max(lo, base), b = min(hi, base + len);
      const uint32_t start = base;
      base += len;
      if (a >= b) continue;
      for (uint32_t s = s0 + (a - start) + threadIdx.x; s < s0 + (b - start); s += blockDim.x) {
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
          const float2 *bp = region + ((q - q0) * R + iv_rel) * RS + iu_rel;
          float pr = 0.f, pi = 0.f;
#pragma unroll
          for (int j = 0; j < kMaxSupport; ++j) {
            if (j < W) {
              const float2 *rowp = bp + j * RS;
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
          }
          sr += kw * pr;
          si += kw * pi;
        }
        atomicAdd(&acc[s], make_float2(sr, si));
      }
    }
    __syncthreads();
  }
}

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    WGPU_CUDA(cudaGetDevice(&dev));
    WGPU_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  }
  return n;
}

// Plans the work items of one batch: scanned item offsets (n_units + 1) and
// the item -> unit descriptors.  Returns the number of items (one small
// device-to-host read that sizes the launch).
template <int T, int G>
uint32_t plan_items(DeviceArena &arena, const DevPlan &p, const uint32_t *off, int p_begin,
                    int n_batch, bool degrid, float2 *planes, uint32_t **item_off,
                    uint32_t **desc, cudaStream_t s) {
  const int n_groups = (n_batch + G - 1) / G;
  const int n_units = p.ntu * p.ntv * n_groups;
  *item_off = (uint32_t *)arena.get(kSlotItems, sizeof(uint32_t) * (2 * (size_t)n_units + 4));
  uint32_t *counts = *item_off + n_units + 2;
  const int warps_per_block = kThreads / 32;
  const unsigned blocks = (unsigned)((n_units + warps_per_block - 1) / warps_per_block);
  grid_plan_kernel<T, G><<<blocks, kThreads, 0, s>>>(p, off, p_begin, n_batch, n_units,
                                                     degrid ? 1 : 0, *item_off, counts, planes);
  check_launch("grid_plan_kernel");
  WGPU_CUDA(cudaMemsetAsync(*item_off + n_units, 0, sizeof(uint32_t), s));
  exclusive_scan_u32(arena, *item_off, n_units + 1, s);
  uint32_t *pinned = (uint32_t *)arena.get(kSlotCounter, 64);
  uint32_t total = 0;
  WGPU_CUDA(cudaMemcpyAsync(&total, *item_off + n_units, sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaStreamSynchronize(s));
  (void)pinned;
  *desc = (uint32_t *)arena.get(kSlotItemDesc, sizeof(uint32_t) * ((size_t)total + 1));
  fill_items_kernel<<<(n_units + 255) / 256, 256, 0, s>>>(*item_off, counts, n_units, *desc);
  check_launch("fill_items_kernel");
  return total;
}

template <int T, int G>
void grid_batch(DeviceArena &arena, const DevPlan &p, const VisRecord *rec,
                const uint32_t *off, int p_begin, int n_batch, float2 *planes,
                cudaStream_t s) {
  uint32_t *item_off, *desc;
  const uint32_t total =
      plan_items<T, G>(arena, p, off, p_begin, n_batch, false, planes, &item_off, &desc, s);
  if (total == 0) return;
  int per_sm = 0;
  WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grid_kernel<T, G>, kThreads, 0));
  const uint32_t blocks = std::min<uint32_t>(total, (uint32_t)(sm_count() * std::max(per_sm, 1)));
  grid_kernel<T, G><<<blocks, kThreads, 0, s>>>(p, rec, off, p_begin, n_batch, item_off, desc,
                                                total, planes);
  check_launch("grid_kernel");
}

template <int T, int G>
void degrid_batch(DeviceArena &arena, const DevPlan &p, const VisRecord *rec,
                  const uint32_t *off, int p_begin, int n_batch, const float2 *planes,
                  float2 *acc, cudaStream_t s) {
  uint32_t *item_off, *desc;
  const uint32_t total =
      plan_items<T, G>(arena, p, off, p_begin, n_batch, true, nullptr, &item_off, &desc, s);
  if (total == 0) return;
  const int R = T + p.support - 1;
  const size_t smem = sizeof(float2) * G * R * (R + 1);
  WGPU_CUDA(cudaFuncSetAttribute(degrid_kernel<T, G>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, degrid_kernel<T, G>,
                                                          kThreads, smem));
  const uint32_t blocks = std::min<uint32_t>(total, (uint32_t)(sm_count() * std::max(per_sm, 1)));
  degrid_kernel<T, G><<<blocks, kThreads, smem, s>>>(p, rec, off, p_begin, n_batch, item_off,
                                                     desc, total, planes, acc);
  check_launch("degrid_kernel");
}

}  // namespace

int grid_plane_group() { return 4; }

void launch_grid(DeviceArena &arena, const DevPlan &p, const VisRecord *rec,
                 const uint32_t *off, int p_begin, int n_batch, float2 *planes,
                 cudaStream_t s) {
  if (p.tile == 32)
    grid_batch<32, 4>(arena, p, rec, off, p_begin, n_batch, planes, s);
  else if (p.tile == 16)
    grid_batch<16, 8>(arena, p, rec, off, p_begin, n_batch, planes, s);
  else
    throw Error(WGPU_ERR_INVALID, "tile must be 16 or 32");
}

void launch_degrid(DeviceArena &arena, const DevPlan &p, const VisRecord *rec,
                   const uint32_t *off, int p_begin, int n_batch, const float2 *planes,
                   float2 *acc, cudaStream_t s) {
  if (p.tile == 32)
    degrid_batch<32, 4>(arena, p, rec, off, p_begin, n_batch, planes, acc, s);
  else if (p.tile == 16)
    degrid_batch<16, 8>(arena, p, rec, off, p_begin, n_batch, planes, acc, s);
  else
    throw Error(WGPU_ERR_INVALID, "tile must be 16 or 32");
}

}  // namespace wgpu
