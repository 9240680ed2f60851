// K2 gridding and K3 degridding over (uv tile, w-plane group) work units.
//
// Work unit = (uv tile T x T, group of G consecutive w planes).  A unit reads
// the visibilities bucketed in its own tile (footprint corner in the tile;
// the key's class says which neighbours the footprint reaches), restricted by
// key range to the first planes that reach the group.  Units are split into
// work items of at most kItemVis visibility reads, and one persistent launch
// works through the items of a plane batch, so that the crowded tiles of a
// dense uv core are shared by many CTAs.
//
// Gridding item: a block accumulates whole footprints into the unit's halo
// region (the tile plus W - 1 cells to the right and up, G planes) in shared
// memory; warp k owns the halo rows congruent to k modulo 8, so every row of a
// footprint has one owner and cells are updated with plain read-add-writes.
// The tile's own cells are written to the planes once per item; the border
// cells go to the unit's spill slot and a fix-up pass adds them into the
// neighbouring tiles.  One launch can also serve many jobs (facets x channel
// groups), each with its own plan, records and planes (grid_kernel_multi).
//
// Degridding item: loads its tile plus a (W-1)-cell halo of G planes into
// shared memory and gathers, for each visibility of its slice of the own
// bucket, the W x W x (planes in the group) weighted sum, added to the
// per-visibility accumulator.
#include <algorithm>

#include "tma.cuh"
#include "wgpu_internal.h"

namespace wgpu {

namespace {

constexpr int kThreads = 256;
constexpr uint32_t kItemVis = 2048;  // visibility reads per work item
constexpr int kTile = 16;            // uv tile edge (cells)
constexpr int kGridPlanes = 16;      // w planes per gridding work unit

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
// and up, 3 up).  A unit reads the four class ranges of its own tile (entries
// 0-3 below), each restricted to first planes that reach the plane group; the
// remaining entries name the left, lower and lower-left neighbours' ranges
// that reach a tile.
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

// Planning pass: one warp per unit counts the reads of the unit (the four
// classes of its own tile) and its work items.
template <int T, int G>
__global__ void __launch_bounds__(kThreads)
    grid_plan_kernel(DevPlan p, const uint32_t *__restrict__ off, int p_begin, int n_batch,
                     int n_units, int degrid, uint32_t *__restrict__ items,
                     uint32_t *__restrict__ counts) {
  const int unit = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (unit >= n_units) return;
  const int n_tiles = p.ntu * p.ntv;
  const int tile = unit % n_tiles, group = unit / n_tiles;
  const int q0 = p_begin + group * G;
  const int q1 = min(q0 + G, p_begin + n_batch);
  uint32_t cnt = 0;
  if (lane < 4) {
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
}

// Spill slots: flags of the units with visibilities (scanned afterwards), then
// slot = scanned index for those units and -1 for the others.
__global__ void slot_flags_kernel(const uint32_t *__restrict__ counts, int n_units,
                                  uint32_t *__restrict__ flags) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u < n_units) flags[u] = counts[u] > 0 ? 1u : 0u;
  if (u == n_units) flags[u] = 0u;
}
__global__ void slot_final_kernel(const uint32_t *__restrict__ counts, int n_units,
                                  int *__restrict__ slot) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u < n_units && counts[u] == 0) slot[u] = -1;
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

// Geometry of the gridding halo region: R = T + W - 1 rows and columns; the
// plane stride is padded to 8 modulo 16 float2 for W <= 8 (a half-warp then
// covers eight columns of two planes on distinct bank pairs); G planes per
// unit (16 for W <= 8, 8 above, to keep the region near 70 KB).
__host__ __device__ constexpr int grid_group(int W) { return W <= 8 ? 16 : 8; }
__host__ __device__ constexpr int halo_rows(int T, int W) { return T + W - 1; }
__host__ __device__ constexpr int halo_plane(int T, int W) {
  return W <= 8 ? ((halo_rows(T, W) * halo_rows(T, W) + 15) / 16 * 16 + 8)
                : ((halo_rows(T, W) * halo_rows(T, W) + 15) / 16 * 16);
}
// Border cells of a unit (outside its tile): the right strip (columns T..R-1,
// all R rows), then the top strip (rows T..R-1, columns 0..T-1).
__host__ __device__ constexpr int spill_cells(int T, int W) {
  return (W - 1) * halo_rows(T, W) + (W - 1) * T;
}
// A unit's spill slot: its G planes' border cells, then one cell whose first
// word is the mask of the planes the slot holds (bit q: plane q of the group
// was written; the fix-up reads no other plane).
__host__ __device__ constexpr int slot_cells(int G, int B) { return G * B + 1; }
__host__ __device__ __forceinline__ int border_index(int T, int W, int r, int c) {
  return c >= T ? r * (W - 1) + (c - T) : (W - 1) * halo_rows(T, W) + (r - T) * T + c;
}

// Shared-memory layout of the gridding kernels: the halo cells [G][plane],
// then the staged round: the meta data of each read (int4: u and v corner
// relative to the tile, first plane relative to the group, and the range
// [lo, hi) of footprint planes inside the group as lo | hi << 8), the
// visibility times the w kernel value of each footprint plane
// ([kGridRound][W] float2), and the u, v kernel values [kGridRound][kw] with
// kw = 2W rounded up to an odd count (the odd stride keeps the stores of a warp
// on distinct banks).
constexpr int kGridRound = 32;  // records staged per round (eight threads stage each)
__host__ __device__ constexpr int grid_weight_stride(int W) { return (2 * W) | 1; }
template <int T, int G, int W>
constexpr size_t grid_smem_bytes() {
  return sizeof(float2) * G * halo_plane(T, W) +
         (size_t)kGridRound * (sizeof(int4) + sizeof(float2) * W +
                               sizeof(float) * grid_weight_stride(W));
}

// Shared memory of the gridding kernels (see grid_smem_bytes).
struct GridSmem {
  float2 *cells;  // [G][halo plane]
  int4 *meta;     // (iu_rel, iv_rel, ip_rel, lo | hi << 8) per staged read
  float2 *vz;     // [kGridRound][W]: visibility times kz[dz]
  float *wts;     // [kGridRound][kw]: kx[W], ky[W]
  uint32_t *rs0, *rcum;
};

template <int T, int G, int W>
__device__ __forceinline__ GridSmem grid_smem(float4 *smem4, uint32_t *rs0, uint32_t *rcum) {
  GridSmem sm;
  sm.cells = reinterpret_cast<float2 *>(smem4);
  sm.meta = reinterpret_cast<int4 *>(sm.cells + G * halo_plane(T, W));
  sm.vz = reinterpret_cast<float2 *>(sm.meta + kGridRound);
  sm.wts = reinterpret_cast<float *>(sm.vz + kGridRound * W);
  sm.rs0 = rs0;
  sm.rcum = rcum;
  return sm;
}

// One gridding work item (descriptor d, item index `item` of its batch).  The
// halo cells are zero on entry and on return; ends with a block barrier
// unless the unit has no visibilities.  Reads are staged in rounds of
// kGridRound with their kernel values (evaluated once per read by eight
// threads); every warp then adds, for every read of the round, the footprint
// row it owns (rows congruent to the warp index modulo 8): lanes cover
// (footprint column, plane lane) and step through the footprint's planes.
template <int T, int G, int W>
__device__ __forceinline__ void grid_item(const DevPlan &p, const VisRecord *__restrict__ rec,
                                          const uint32_t *__restrict__ off, int p_begin,
                                          int n_batch, const uint32_t *__restrict__ item_off,
                                          const int *__restrict__ slots, float2 *__restrict__ spill,
                                          uint32_t d, uint32_t item,
                                          float2 *__restrict__ planes, const GridSmem &sm) {
  constexpr int kCols = W <= 8 ? 8 : 16;          // lanes across footprint columns
  constexpr int kPlaneLanes = 32 / kCols;         // 4 (W <= 8) or 2
  constexpr int kSteps = (W + kPlaneLanes - 1) / kPlaneLanes;
  constexpr int kWS = grid_weight_stride(W);
  constexpr int R = halo_rows(T, W);
  constexpr int PS = halo_plane(T, W);
  constexpr int B = spill_cells(T, W);
  float2 *cells = sm.cells;
  float *wts = sm.wts;
  uint32_t *rs0 = sm.rs0, *rcum = sm.rcum;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ci = lane % kCols;       // footprint column offset
  const int pl = lane / kCols;       // plane lane
  const float inv_half = 2.0f / (float)W;
  const int n_tiles = p.ntu * p.ntv;
  const size_t plane_elems = (size_t)p.nu * p.nv;
  const int unit = (int)(d & 0x7fffffffu);
  const int tile = unit % n_tiles, group = unit / n_tiles;
  const int tu = tile % p.ntu, tv = tile / p.ntu;
  const int q0 = p_begin + group * G;
  const int q1 = min(q0 + G, p_begin + n_batch);
  const int nq = q1 - q0;
  if (d & 0x80000000u) {
    // no visibility reaches this unit: its own cells are zero
    for (int c = threadIdx.x; c < nq * T * T; c += kThreads) {
      const int pq = c / (T * T), rem = c - pq * (T * T);
      const int rr = rem / T, cc = rem - rr * T;
      planes[(size_t)(q0 + pq - p_begin) * plane_elems + (size_t)(tv * T + rr) * p.nu +
             tu * T + cc] = make_float2(0.f, 0.f);
    }
    return;
  }
  const uint32_t first = __ldg(item_off + unit);
  const uint32_t n_items = __ldg(item_off + unit + 1) - first;
  if (threadIdx.x < 4) {
    uint32_t a, b;
    unit_range(p, off, tile, q0, q1, threadIdx.x, &a, &b);
    rs0[threadIdx.x] = a;
    rcum[threadIdx.x + 1] = b - a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    rcum[0] = 0;
    for (int r = 0; r < 4; ++r) rcum[r + 1] += rcum[r];
  }
  __syncthreads();
  const uint32_t lo = (item - first) * kItemVis;
  const uint32_t hi = min(lo + kItemVis, rcum[4]);

  for (uint32_t rb = lo; rb < hi; rb += kGridRound) {
    // stage: eight threads share read t; roles 0-3 evaluate half of kx or ky
    // each, roles 4-5 half of the visibility times kz, role 6 writes the meta
    // data
    {
      static_assert(kThreads == 8 * kGridRound, "eight staging roles");
      constexpr int kHalf = (W + 1) / 2;
      const int t = threadIdx.x % kGridRound;
      const int role = threadIdx.x / kGridRound;
      const uint32_t pos = rb + (uint32_t)t;
      if (pos < hi && role < 7) {
        int r = 0;
        while (pos >= rcum[r + 1]) ++r;
        const VisRecord v = load_record(rec + rs0[r] + (pos - rcum[r]));
        float *w = wts + t * kWS;
        if (role < 4) {
          const int dim = role >> 1, k0 = (role & 1) * kHalf;
          const float f = dim == 0 ? v.fu : v.fv;
#pragma unroll
          for (int kk = 0; kk < kHalf; ++kk) {
            const int k = k0 + kk;
            if (k < W) w[dim * W + k] = es_eval(p.beta, (f + (float)k) * inv_half);
          }
        } else if (role < 6) {
          const int k0 = (role & 1) * kHalf;
          float2 *vz = sm.vz + t * W;
#pragma unroll
          for (int kk = 0; kk < kHalf; ++kk) {
            const int k = k0 + kk;
            if (k < W) {
              const float kz = p.n_planes == 1 ? (k == 0 ? 1.0f : 0.0f)
                                               : es_eval(p.beta, (v.fw + (float)k) * inv_half);
              // W = 8: plane k = s * 4 + pl at (pl, s), so that a lane's two
              // planes are one 16-byte load
              const int at = W == 8 ? ((k & 3) * 2 + (k >> 2)) : k;
              vz[at] = make_float2(v.re * kz, v.im * kz);
            }
          }
        } else {
          // own-tile records: the corner lies in the tile (0 <= rel < T);
          // footprint planes dz in [lo, hi) fall inside the group
          const int ip_rel = v.ip - q0;
          const int lo = max(0, -ip_rel), hi = min(W, nq - ip_rel);
          sm.meta[t] = make_int4(v.iu - tu * T, v.iv - tv * T, ip_rel, lo | (hi << 8));
        }
      }
    }
    __syncthreads();
    const int n_round = (int)min((uint32_t)kGridRound, hi - rb);
    for (int m = 0; m < n_round; ++m) {
      const int4 mt = sm.meta[m];  // (iu_rel, iv_rel, ip_rel, lo | hi << 8)
      const float *w = wts + m * kWS;
      const float2 *vz = sm.vz + m * W;
      const int lo = mt.w & 255, n_dz = (mt.w >> 8) - lo;
      // the footprint's cells of plane ip_rel (dz = 0); the range test keeps
      // every access inside the group's planes
      const int col = mt.z * PS + mt.x + ci;
      // footprint rows owned by this warp: dv = (warp - iv_rel) mod 8, + 8
      auto add_row = [&](int dv) {
        const float wuv = w[ci] * w[W + dv];
        float2 *cb = cells + (mt.y + dv) * R + col;
        if constexpr (W == 8) {
          // planes pl and pl + 4 of this lane in one load
          const float4 z2 = reinterpret_cast<const float4 *>(vz)[pl];
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            const int dz = s * 4 + pl;
            if ((unsigned)(dz - lo) < (unsigned)n_dz) {
              const float zx = s == 0 ? z2.x : z2.z, zy = s == 0 ? z2.y : z2.w;
              float2 c = cb[dz * PS];
              c.x = fmaf(wuv, zx, c.x);
              c.y = fmaf(wuv, zy, c.y);
              cb[dz * PS] = c;
            }
          }
        } else {
#pragma unroll
          for (int s = 0; s < kSteps; ++s) {
            const int dz = s * kPlaneLanes + pl;
            if ((unsigned)(dz - lo) < (unsigned)n_dz) {
              const float2 z = vz[dz];
              float2 c = cb[dz * PS];
              c.x = fmaf(wuv, z.x, c.x);
              c.y = fmaf(wuv, z.y, c.y);
              cb[dz * PS] = c;
            }
          }
        }
      };
      if constexpr (W == 8) {
        add_row((warp - mt.y) & 7);  // one row per warp, every lane's column inside
      } else {
        for (int dv = (warp - mt.y) & 7; dv < W; dv += 8)
          if (ci < W) add_row(dv);
      }
      __syncwarp();  // the next read's lanes may update the same cells
    }
    __syncthreads();
  }
  // flush: the tile's cells to the planes (a split unit adds into cells
  // zeroed beforehand), the border cells to the unit's spill slot
  const int slot = __ldg(slots + unit);
  float2 *sp = spill + (size_t)slot * slot_cells(G, B);
  if (threadIdx.x == 0) {
    unsigned *mask = reinterpret_cast<unsigned *>(sp + G * B);
    const unsigned all = (1u << nq) - 1u;
    if (n_items == 1)
      *mask = all;
    else
      atomicOr(mask, all);
  }
  for (int c = threadIdx.x; c < nq * R * R; c += kThreads) {
    const int pq = c / (R * R), rem = c - pq * (R * R);
    const int rr = rem / R, cc = rem - rr * R;
    float2 *src = cells + pq * PS + rr * R + cc;
    const float2 val = *src;
    *src = make_float2(0.f, 0.f);
    float2 *dst;
    if (rr < T && cc < T)
      dst = planes + (size_t)(q0 + pq - p_begin) * plane_elems + (size_t)(tv * T + rr) * p.nu +
            tu * T + cc;
    else
      dst = sp + (size_t)pq * B + border_index(T, W, rr, cc);
    if (n_items == 1)
      *dst = val;
    else
      atomicAdd(dst, val);
  }
  __syncthreads();
}

// ---- gridding by corner runs (W <= 8) -------------------------------------
//
// The bucketing orders the samples of every (tile, class, first plane) key by
// their footprint corner inside the tile, so the samples that share an exact
// corner (iu, iv, ip) are consecutive; in the wide-field workload half of the
// samples lie in runs of eight or more.  A warp takes a contiguous chunk of
// the item's reads and holds a whole 8 x 8 x 8 footprint in registers: lane l
// owns footprint column i = l % 8, rows j = l / 8 and l / 8 + 4, and all eight
// planes (16 complex accumulators).  Each read adds its kernel-weighted
// visibility to the accumulators; only when the corner changes (and at the
// end of the chunk) does the warp add the footprint into the halo, with
// shared-memory atomics because the warps' footprints may overlap.  Kernel
// values are evaluated once per read by the lane that stages it (eight
// values along each axis; the w values already multiplied by the visibility).
//
// The halo holds fixed-point integers: a run's float sums are scaled by
// S = 2^30 / sum over the item's reads of (|re| + |im|), rounded and added
// with native integer atomics, and converted back when the halo is written
// out.  Every kernel value is at most one, so no cell component can exceed
// 2^30 (no overflow), and the integer sums are exact and independent of the
// order in which the warps add them.  Each flush rounds by at most half a
// unit, i.e. 2^-31 of the item's summed magnitude; an item holds at most 2048
// reads, which bounds that step.
constexpr int kRunWarps = kThreads / 32;
constexpr int kRunBatch = 32;  // reads staged per warp at a time
struct __align__(16) RunStage {
  float kx[8];    // u kernel values (zero beyond W)
  float2 ky2[4];  // (ky[j], ky[j + 4])
  float2 vz[8];   // visibility times the w kernel value of footprint plane k
  int meta;       // iu_rel | iv_rel << 8 | (ip_rel + 128) << 16
  int pad[3];
};
static_assert(sizeof(RunStage) == 144, "run stage layout");

template <int T, int G, int W>
constexpr size_t grid_runs_smem_bytes() {
  return sizeof(float2) * G * halo_plane(T, W) + sizeof(RunStage) * kRunWarps * kRunBatch;
}

// The footprint of the current run (corner `meta`) into the fixed-point halo
// cells of the group's planes, scaled by `scale`.
template <int T, int G, int W>
__device__ __forceinline__ void run_flush(int2 *cells, int meta, int nq, int i, int jb,
                                          float scale, const float2 (&acc)[2][8]) {
  constexpr int R = halo_rows(T, W);
  constexpr int PS = halo_plane(T, W);
  const int iu_rel = meta & 255, iv_rel = (meta >> 8) & 255, ip_rel = (meta >> 16) - 128;
  if (i >= W) return;
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const int j = jb + 4 * t;
    if (j >= W) continue;
    int2 *row = cells + (iv_rel + j) * R + iu_rel + i;
#pragma unroll
    for (int k = 0; k < W; ++k) {
      const int z = ip_rel + k;
      if (z >= 0 && z < nq) {
        int2 *c = row + z * PS;
        atomicAdd(&c->x, __float2int_rn(acc[t][k].x * scale));
        atomicAdd(&c->y, __float2int_rn(acc[t][k].y * scale));
      }
    }
  }
}

template <int T, int G, int W>
__device__ __forceinline__ void grid_item_runs(const DevPlan &p, const VisRecord *__restrict__ rec,
                                               const uint32_t *__restrict__ off, int p_begin,
                                               int n_batch, const uint32_t *__restrict__ item_off,
                                               const int *__restrict__ slots,
                                               float2 *__restrict__ spill, uint32_t d,
                                               uint32_t item, float2 *__restrict__ planes,
                                               int2 *cells, RunStage *stage, uint32_t *rs0,
                                               uint32_t *rcum, float *red, int *prange) {
  static_assert(W <= 8, "runs gridding holds an 8 x 8 x 8 footprint");
  static_assert(kThreads == T * T, "one thread per tile cell in the write-out");
  constexpr int R = halo_rows(T, W);
  constexpr int PS = halo_plane(T, W);
  constexpr int B = spill_cells(T, W);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = lane & 7, jb = lane >> 3;
  const float inv_half = 2.0f / (float)W;
  const int n_tiles = p.ntu * p.ntv;
  const size_t plane_elems = (size_t)p.nu * p.nv;
  const int unit = (int)(d & 0x7fffffffu);
  const int tile = unit % n_tiles, group = unit / n_tiles;
  const int tu = tile % p.ntu, tv = tile / p.ntu;
  const int q0 = p_begin + group * G;
  const int q1 = min(q0 + G, p_begin + n_batch);
  const int nq = q1 - q0;
  if (d & 0x80000000u) {
    // no visibility reaches this unit: its own cells are zero
    for (int c = threadIdx.x; c < nq * T * T; c += kThreads) {
      const int pq = c / (T * T), rem = c - pq * (T * T);
      const int rr = rem / T, cc = rem - rr * T;
      planes[(size_t)(q0 + pq - p_begin) * plane_elems + (size_t)(tv * T + rr) * p.nu +
             tu * T + cc] = make_float2(0.f, 0.f);
    }
    return;
  }
  const uint32_t first = __ldg(item_off + unit);
  const uint32_t n_items = __ldg(item_off + unit + 1) - first;
  if (threadIdx.x < 4) {
    uint32_t a, b;
    unit_range(p, off, tile, q0, q1, threadIdx.x, &a, &b);
    rs0[threadIdx.x] = a;
    rcum[threadIdx.x + 1] = b - a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    rcum[0] = 0;
    for (int r = 0; r < 4; ++r) rcum[r + 1] += rcum[r];
  }
  __syncthreads();
  const uint32_t lo = (item - first) * kItemVis;
  const uint32_t hi = min(lo + kItemVis, rcum[4]);
  // fixed-point scale of the halo: 2^30 over the item's summed magnitudes
  // (with a margin for the float sum and kernel values rounded above one)
  // and the range of the group's planes the item's footprints touch (first
  // planes ip_lo..ip_hi, footprints W planes deep)
  int ip_lo = 0x7fffffff, ip_hi = -0x7fffffff;
  {
    float part = 0.f;
    for (uint32_t pos = lo + threadIdx.x; pos < hi; pos += kThreads) {
      int r = 0;
      while (pos >= rcum[r + 1]) ++r;
      const VisRecord *vr = rec + rs0[r] + (pos - rcum[r]);
      const float2 v = __ldg(reinterpret_cast<const float2 *>(vr));
      const int ip = __ldg(&vr->ip);
      part += fabsf(v.x) + fabsf(v.y);
      ip_lo = min(ip_lo, ip);
      ip_hi = max(ip_hi, ip);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    ip_lo = __reduce_min_sync(0xffffffffu, ip_lo);
    ip_hi = __reduce_max_sync(0xffffffffu, ip_hi);
    if (lane == 0) {
      red[warp] = part;
      atomicMin(&prange[0], ip_lo);
      atomicMax(&prange[1], ip_hi);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      float sum = 0.f;
      for (int w = 0; w < kRunWarps; ++w) sum += red[w];
      red[kRunWarps] = sum > 0.f ? 1073741824.0f / (sum * 1.001f) : 1.0f;
    }
    __syncthreads();
  }
  const float scale = red[kRunWarps];
  // planes [z_lo, z_hi) of the group hold this item's footprints
  const int z_lo = max(prange[0] - q0, 0), z_hi = min(prange[1] - q0 + W, nq);
  // this warp's contiguous chunk of the item's reads
  const uint32_t per = (hi - lo + kRunWarps - 1) / kRunWarps;
  const uint32_t c0 = min(lo + (uint32_t)warp * per, hi);
  const uint32_t c1 = min(c0 + per, hi);
  RunStage *ws = stage + warp * kRunBatch;
  float2 acc[2][8];
#pragma unroll
  for (int t = 0; t < 2; ++t)
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[t][k] = make_float2(0.f, 0.f);
  int cur = -1;
  for (uint32_t b0 = c0; b0 < c1; b0 += kRunBatch) {
    __syncwarp();  // the previous batch has been read
    {
      const uint32_t pos = b0 + (uint32_t)lane;
      if (pos < c1) {
        int r = 0;
        while (pos >= rcum[r + 1]) ++r;
        const VisRecord v = load_record(rec + rs0[r] + (pos - rcum[r]));
        RunStage &st = ws[lane];
        float ky[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          st.kx[k] = k < W ? es_eval(p.beta, (v.fu + (float)k) * inv_half) : 0.f;
          ky[k] = k < W ? es_eval(p.beta, (v.fv + (float)k) * inv_half) : 0.f;
          const float kz = k >= W ? 0.f
                           : p.n_planes == 1 ? (k == 0 ? 1.0f : 0.0f)
                                             : es_eval(p.beta, (v.fw + (float)k) * inv_half);
          st.vz[k] = make_float2(v.re * kz, v.im * kz);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) st.ky2[k] = make_float2(ky[k], ky[k + 4]);
        st.meta = (v.iu - tu * T) | ((v.iv - tv * T) << 8) | ((v.ip - q0 + 128) << 16);
      }
    }
    __syncwarp();
    const int n_b = (int)min((uint32_t)kRunBatch, c1 - b0);
    int m = 0;
    while (m < n_b) {
      // a new corner (warp-uniform: every lane reads the same read)
      const int meta = ws[m].meta;
      if (meta != cur) {
        if (cur >= 0) run_flush<T, G, W>(cells, cur, nq, i, jb, scale, acc);
#pragma unroll
        for (int t = 0; t < 2; ++t)
#pragma unroll
          for (int k = 0; k < 8; ++k) acc[t][k] = make_float2(0.f, 0.f);
        cur = meta;
      }
      // the batch's reads of this corner, accumulated in registers
      do {
        const RunStage &st = ws[m];
        const float kx = st.kx[i];
        const float2 ky = st.ky2[jb];
        const float w0 = kx * ky.x, w1 = kx * ky.y;
        // (re, im) pairs in one paired FP32 FMA each (the same roundings as
        // two scalar FMAs)
        const float2 w02 = make_float2(w0, w0), w12 = make_float2(w1, w1);
#pragma unroll
        for (int k = 0; k < W; k += 2) {
          if (k + 1 < W) {
            const float4 z = *reinterpret_cast<const float4 *>(&st.vz[k]);
            const float2 za = make_float2(z.x, z.y), zb = make_float2(z.z, z.w);
            acc[0][k] = __ffma2_rn(w02, za, acc[0][k]);
            acc[1][k] = __ffma2_rn(w12, za, acc[1][k]);
            acc[0][k + 1] = __ffma2_rn(w02, zb, acc[0][k + 1]);
            acc[1][k + 1] = __ffma2_rn(w12, zb, acc[1][k + 1]);
          } else {
            const float2 z = st.vz[k];
            acc[0][k] = __ffma2_rn(w02, z, acc[0][k]);
            acc[1][k] = __ffma2_rn(w12, z, acc[1][k]);
          }
        }
        ++m;
      } while (m < n_b && ws[m].meta == cur);
    }
  }
  if (cur >= 0) run_flush<T, G, W>(cells, cur, nq, i, jb, scale, acc);
  __syncthreads();
  // write-out, plane by plane: the tile's T x T cells to the planes (one per
  // thread; a split unit adds into cells zeroed beforehand), the border cells
  // to the unit's spill slot in spill order (border_index); the halo is left
  // zero
  const float inv = 1.0f / scale;
  const bool add = n_items > 1;
  const int slot = __ldg(slots + unit);
  float2 *sp = spill + (size_t)slot * slot_cells(G, B);
  const int tr = threadIdx.x / T, tc = threadIdx.x % T;
  if (threadIdx.x == 0) {
    unsigned *mask = reinterpret_cast<unsigned *>(sp + G * B);
    const unsigned bits = z_hi > z_lo ? ((1u << z_hi) - 1u) & ~((1u << z_lo) - 1u) : 0u;
    if (add)
      atomicOr(mask, bits);
    else
      *mask = bits;
    prange[0] = 0x7fffffff;  // for the block's next item (read before the barrier above)
    prange[1] = -0x7fffffff;
  }
  for (int pq = 0; pq < nq; ++pq) {
    if (pq < z_lo || pq >= z_hi) {
      // a plane the item does not touch: its halo cells are zero; the unit's
      // own cells get zeros unless a split unit's were zeroed beforehand, and
      // its spill is not written (the mask leaves it out)
      if (!add)
        planes[(size_t)(q0 + pq - p_begin) * plane_elems + (size_t)(tv * T + tr) * p.nu +
               tu * T + tc] = make_float2(0.f, 0.f);
      continue;
    }
    int2 *cp = cells + pq * PS;
    {
      int2 *src = cp + tr * R + tc;
      const int2 q = *src;
      *src = make_int2(0, 0);
      const float2 val = make_float2((float)q.x * inv, (float)q.y * inv);
      float2 *dst = planes + (size_t)(q0 + pq - p_begin) * plane_elems +
                    (size_t)(tv * T + tr) * p.nu + tu * T + tc;
      if (add)
        atomicAdd(dst, val);
      else
        *dst = val;
    }
    float2 *spq = sp + (size_t)pq * B;
    for (int b = threadIdx.x; b < B; b += kThreads) {
      int rr, cc;
      if (b < (W - 1) * R) {
        rr = b / (W - 1);
        cc = T + b - rr * (W - 1);
      } else {
        rr = T + (b - (W - 1) * R) / T;
        cc = (b - (W - 1) * R) % T;
      }
      int2 *src = cp + rr * R + cc;
      const int2 q = *src;
      *src = make_int2(0, 0);
      const float2 val = make_float2((float)q.x * inv, (float)q.y * inv);
      if (add)
        atomicAdd(spq + b, val);
      else
        spq[b] = val;
    }
  }
  __syncthreads();
}

// Shared memory of the gridding kernels: the halo cells and either the
// round-staging of grid_item (W > 8) or the per-warp run staging (W <= 8).
template <int T, int G, int W>
constexpr size_t grid_kernel_smem_bytes() {
  if constexpr (W <= 8)
    return grid_runs_smem_bytes<T, G, W>();
  else
    return grid_smem_bytes<T, G, W>();
}

// One gridding work item with the variant for the support.
template <int T, int G, int W>
__device__ __forceinline__ void grid_item_any(const DevPlan &p, const VisRecord *__restrict__ rec,
                                              const uint32_t *__restrict__ off, int p_begin,
                                              int n_batch, const uint32_t *__restrict__ item_off,
                                              const int *__restrict__ slots,
                                              float2 *__restrict__ spill, uint32_t d,
                                              uint32_t item, float2 *__restrict__ planes,
                                              float4 *smem4, uint32_t *rs0, uint32_t *rcum,
                                              float *red, int *prange) {
  if constexpr (W <= 8) {
    int2 *cells = reinterpret_cast<int2 *>(smem4);
    RunStage *stage = reinterpret_cast<RunStage *>(cells + G * halo_plane(T, W));
    grid_item_runs<T, G, W>(p, rec, off, p_begin, n_batch, item_off, slots, spill, d, item,
                            planes, cells, stage, rs0, rcum, red, prange);
  } else {
    const GridSmem sm = grid_smem<T, G, W>(smem4, rs0, rcum);
    grid_item<T, G, W>(p, rec, off, p_begin, n_batch, item_off, slots, spill, d, item, planes,
                       sm);
  }
}

// Two blocks per SM for the run variant (its shared memory allows two), three
// for the round variant; both fit in 128 registers per thread.
template <int T, int G, int W>
__global__ void __launch_bounds__(kThreads, 2)
    grid_kernel(DevPlan p, const VisRecord *__restrict__ rec,
                const uint32_t *__restrict__ off, int p_begin, int n_batch,
                const uint32_t *__restrict__ item_off, const uint32_t *__restrict__ desc,
                const int *__restrict__ slots, float2 *__restrict__ spill,
                uint32_t total, float2 *__restrict__ planes) {
  static_assert(kThreads == 256, "eight warps own the halo rows modulo 8");
  extern __shared__ float4 smem4[];
  __shared__ uint32_t rs0[4], rcum[5];
  __shared__ float red[kRunWarps + 1];
  __shared__ int prange[2];  // first planes of the current item's reads
  float2 *cells = reinterpret_cast<float2 *>(smem4);
  for (int c = threadIdx.x; c < G * halo_plane(T, W); c += kThreads)
    cells[c] = make_float2(0.f, 0.f);
  if (threadIdx.x == 0) {
    prange[0] = 0x7fffffff;
    prange[1] = -0x7fffffff;
  }
  __syncthreads();
  uint32_t d_next = blockIdx.x < total ? __ldg(desc + blockIdx.x) : 0u;
  for (uint32_t item = blockIdx.x; item < total; item += gridDim.x) {
    const uint32_t d_cur = d_next;  // the next item's descriptor is loaded meanwhile
    if (item + gridDim.x < total) d_next = __ldg(desc + item + gridDim.x);
    grid_item_any<T, G, W>(p, rec, off, p_begin, n_batch, item_off, slots, spill, d_cur, item,
                           planes, smem4, rs0, rcum, red, prange);
  }
}

// Several gridding jobs (facets x channel groups, each with its own plan,
// records and planes but the same kernel support) in one persistent launch:
// item i belongs to the job j with job_base[j] <= i < job_base[j + 1]; the
// block keeps the current job's description in shared memory.
template <int T, int G, int W>
__global__ void __launch_bounds__(kThreads, 2)
    grid_kernel_multi(const GridJob *__restrict__ jobs, const uint32_t *__restrict__ job_base,
                      int n_jobs, uint32_t total) {
  static_assert(kThreads == 256, "eight warps own the halo rows modulo 8");
  static_assert(sizeof(GridJob) % 8 == 0, "job copied in 8-byte words");
  extern __shared__ float4 smem4[];
  __shared__ uint32_t rs0[4], rcum[5];
  __shared__ float red[kRunWarps + 1];
  __shared__ int prange[2];
  __shared__ GridJob job;
  float2 *cells = reinterpret_cast<float2 *>(smem4);
  for (int c = threadIdx.x; c < G * halo_plane(T, W); c += kThreads)
    cells[c] = make_float2(0.f, 0.f);
  if (threadIdx.x == 0) {
    prange[0] = 0x7fffffff;
    prange[1] = -0x7fffffff;
  }
  int cur = -1;
  for (uint32_t item = blockIdx.x; item < total; item += gridDim.x) {
    int lo = 0, hi = n_jobs - 1;  // last job whose base is <= item
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(job_base + mid) <= item) lo = mid; else hi = mid - 1;
    }
    if (lo != cur) {
      __syncthreads();  // nobody reads the previous job any more
      const unsigned long long *src = reinterpret_cast<const unsigned long long *>(jobs + lo);
      unsigned long long *dst = reinterpret_cast<unsigned long long *>(&job);
      for (int k = threadIdx.x; k < (int)(sizeof(GridJob) / 8); k += kThreads) dst[k] = __ldg(src + k);
      cur = lo;
    }
    __syncthreads();
    const uint32_t local = item - __ldg(job_base + lo);
    grid_item_any<T, G, W>(job.p, job.rec, job.off, job.p_begin, job.n_batch, job.item_off,
                           job.slot, job.spill, __ldg(job.desc + local), local, job.planes, smem4,
                           rs0, rcum, red, prange);
  }
}

// Fix-up after a gridding pass: every tile cell within W - 1 of the tile's
// left or lower edge receives the border cells that its left, lower and
// lower-left neighbours spilled (one block per unit, one thread per cell of a
// plane).  Only the planes a neighbour's slot mask names are read; a plane
// that no neighbour wrote is skipped.
__global__ void __launch_bounds__(kThreads)
    spill_fixup_kernel(DevPlan p, int G, int p_begin, int n_batch, int n_units,
                       const int *__restrict__ slots, const float2 *__restrict__ spill,
                       float2 *__restrict__ planes) {
  constexpr int T = kTile;
  static_assert(kThreads == T * T, "one thread per tile cell");
  const int W = p.support, B = (W - 1) * (T + W - 1) + (W - 1) * T;
  const int SC = slot_cells(G, B);
  const int n_tiles = p.ntu * p.ntv;
  const size_t plane_elems = (size_t)p.nu * p.nv;
  const int r = threadIdx.x / T, col = threadIdx.x % T;
  const bool from_left = col < W - 1, from_low = r < W - 1;
  for (int unit = blockIdx.x; unit < n_units; unit += gridDim.x) {
    const int tile = unit % n_tiles, group = unit / n_tiles;
    const int tu = tile % p.ntu, tv = tile / p.ntu;
    const int q0 = p_begin + group * G;
    const int nq = min(q0 + G, p_begin + n_batch) - q0;
    const int tl = (tu + p.ntu - 1) % p.ntu, tb = (tv + p.ntv - 1) % p.ntv;
    const int base = group * n_tiles;
    const int s_left = __ldg(slots + base + tv * p.ntu + tl);
    const int s_low = __ldg(slots + base + tb * p.ntu + tu);
    const int s_diag = __ldg(slots + base + tb * p.ntu + tl);
    auto mask_of = [&](int sl) -> unsigned {
      return sl < 0 ? 0u : __float_as_uint(__ldg(&spill[(size_t)sl * SC + G * B].x));
    };
    const unsigned m_left = mask_of(s_left), m_low = mask_of(s_low), m_diag = mask_of(s_diag);
    const unsigned m_any = m_left | m_low | m_diag;
    if (m_any == 0u || (!from_left && !from_low)) continue;
    for (int pq = 0; pq < nq; ++pq) {
      if (!((m_any >> pq) & 1u)) continue;
      float2 add = make_float2(0.f, 0.f);
      if (from_left && ((m_left >> pq) & 1u)) {
        const float2 v = __ldg(spill + (size_t)s_left * SC + pq * B + border_index(T, W, r, col + T));
        add.x += v.x;
        add.y += v.y;
      }
      if (from_low && ((m_low >> pq) & 1u)) {
        const float2 v = __ldg(spill + (size_t)s_low * SC + pq * B + border_index(T, W, r + T, col));
        add.x += v.x;
        add.y += v.y;
      }
      if (from_left && from_low && ((m_diag >> pq) & 1u)) {
        const float2 v =
            __ldg(spill + (size_t)s_diag * SC + pq * B + border_index(T, W, r + T, col + T));
        add.x += v.x;
        add.y += v.y;
      }
      float2 *dst = planes + (size_t)(q0 + pq - p_begin) * plane_elems +
                    (size_t)(tv * T + r) * p.nu + tu * T + col;
      float2 g = *dst;
      g.x += add.x;
      g.y += add.y;
      *dst = g;
    }
  }
}

// Degridding of one plane batch: the block loads its unit's halo region (the
// tile plus W - 1 cells, G planes) into shared memory as float2 cells with a
// row stride of T + W rounded to 8 mod 16, stages the unit's records in rounds
// and works through them.  W <= 8: groups of eight lanes take one record
// each (lane i sums footprint column i over the rows and planes, a three-step
// shuffle reduction forms the record's sum).  W > 8: one warp per record,
// lanes own footprint cells and a warp-wide reduction forms the sum.
//
// Both stagings are bulk copies (cp.async.bulk, the TMA engine) completing on
// one mbarrier: each halo row is RS cells copied from its plane row (two
// copies where the row wraps around the grid's u edge; every row start is a
// multiple of 16 cells, so every copy is 16-byte aligned), and a round of
// records is at most four contiguous chunks, one per class range.  The waits
// are bounded; a copy that does not complete in time is recorded in *err and
// the block leaves after waiting (bounded) for its copies in flight.
__host__ __device__ constexpr int degrid_row_stride(int R) { return (R + 7) / 16 * 16 + 8; }
template <int T, int G, int W>
constexpr size_t degrid_smem_bytes() {
  return sizeof(float2) * G * (T + W - 1) * degrid_row_stride(T + W - 1);
}

// Blocks per SM that the shared memory allows (five for W <= 8, three above);
// the register cap keeps them
template <int T, int G, int W>
__global__ void __launch_bounds__(kThreads, W <= 8 ? 5 : 3)
    degrid_kernel(DevPlan p, const VisRecord *__restrict__ rec,
                  const uint32_t *__restrict__ off, int p_begin, int n_batch,
                  const uint32_t *__restrict__ item_off, const uint32_t *__restrict__ desc,
                  uint32_t total, const float2 *__restrict__ planes,
                  float2 *__restrict__ acc, unsigned *__restrict__ err) {
  constexpr int R = T + W - 1;
  constexpr int RS = degrid_row_stride(R);
  constexpr int kPlane = R * RS;
  constexpr int kFoot = W * W;
  constexpr int kLaneCells = (kFoot + 31) / 32;
  static_assert((RS * sizeof(float2)) % 16 == 0, "halo rows are whole 16-byte units");
  extern __shared__ __align__(16) float2 halo[];  // [G][R][RS]
  __shared__ uint32_t rs0[4], rcum[5];
  __shared__ __align__(16) float4 stage[kThreads][2];
  __shared__ uint32_t stage_s[kThreads];
  __shared__ __align__(8) uint64_t bar;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float inv_half = 2.0f / (float)W;
  const int n_tiles = p.ntu * p.ntv;
  const size_t plane_elems = (size_t)p.nu * p.nv;
  if (threadIdx.x == 0) {
    mbar_init(&bar);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t phase = 0;
  // waits for the current phase of the staging barrier; false: the copies did
  // not complete in time (recorded once per block, after which the block
  // waits once more for them and stops)
  auto staged = [&]() -> bool {
    const bool ok = mbar_wait_bounded(&bar, phase);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicAdd(err, 1u);
      mbar_wait_bounded(&bar, phase);
      return false;
    }
    phase ^= 1u;
    return true;
  };

  // each item's descriptor is loaded one item ahead, so that the halo copies
  // can be issued as soon as the item starts
  uint32_t d_next = blockIdx.x < total ? __ldg(desc + blockIdx.x) : 0u;
  for (uint32_t item = blockIdx.x; item < total; item += gridDim.x) {
    const uint32_t d_cur = d_next;
    if (item + gridDim.x < total) d_next = __ldg(desc + item + gridDim.x);
    const int unit = (int)(d_cur & 0x7fffffffu);
    const int tile = unit % n_tiles, group = unit / n_tiles;
    const int tu = tile % p.ntu, tv = tile / p.ntu;
    const int q0 = p_begin + group * G;
    const int q1 = min(q0 + G, p_begin + n_batch);
    const uint32_t lo = (item - __ldg(item_off + unit)) * kItemVis;

    const int nq = q1 - q0;
    // halo: warp 0 copies the nq x R rows of RS cells; the first cell of a
    // row is at u = tu * T, and the copy wraps to u = 0 at the grid's edge
    if (warp == 0) {
      const int gu = tu * T;
      const int seg1 = min(RS, p.nu - gu), seg2 = RS - seg1;
      if (lane == 0) {
        fence_proxy_async();
        mbar_expect_tx(&bar, (uint32_t)(nq * R * RS * sizeof(float2)));
      }
      __syncwarp();
      for (int k = lane; k < nq * R; k += 32) {
        const int pq = k / R, r = k - pq * R;
        int gv = tv * T + r;
        if (gv >= p.nv) gv -= p.nv;
        const float2 *row = planes + (size_t)(q0 + pq - p_begin) * plane_elems + (size_t)gv * p.nu;
        float2 *dst = halo + pq * kPlane + r * RS;
        bulk_copy_g2s(dst, row + gu, (uint32_t)(seg1 * sizeof(float2)), &bar);
        if (seg2 > 0) bulk_copy_g2s(dst + seg1, row, (uint32_t)(seg2 * sizeof(float2)), &bar);
      }
    }
    if (threadIdx.x < 4) {
      uint32_t a, b;
      unit_range(p, off, tile, q0, q1, threadIdx.x, &a, &b);
      rs0[threadIdx.x] = a;
      rcum[threadIdx.x + 1] = b - a;
    }
    if (!staged()) return;
    if (threadIdx.x == 0) {
      rcum[0] = 0;
      for (int r = 0; r < 4; ++r) rcum[r + 1] += rcum[r];
    }
    __syncthreads();
    const uint32_t hi = min(lo + kItemVis, rcum[4]);

    for (uint32_t rb = lo; rb < hi; rb += kThreads) {
      const uint32_t re = min(rb + (uint32_t)kThreads, hi);
      // the round's records: one bulk copy per class range it overlaps
      if (threadIdx.x == 0) {
        fence_proxy_async();
        mbar_expect_tx(&bar, (re - rb) * (uint32_t)sizeof(VisRecord));
        for (int r = 0; r < 4; ++r) {
          const uint32_t a = max(rb, rcum[r]), b = min(re, rcum[r + 1]);
          if (a < b)
            bulk_copy_g2s(&stage[a - rb][0], rec + rs0[r] + (a - rcum[r]),
                          (b - a) * (uint32_t)sizeof(VisRecord), &bar);
        }
      }
      {
        const uint32_t pos = rb + threadIdx.x;
        if (pos < re) {
          int r = 0;
          while (pos >= rcum[r + 1]) ++r;
          stage_s[threadIdx.x] = rs0[r] + (pos - rcum[r]);
        }
      }
      if (!staged()) return;
      const int n_round = (int)min((uint32_t)kThreads, hi - rb);
      if constexpr (W <= 8) {
        // groups of eight lanes, one record each: lane i of a group owns
        // footprint column i and sums its W rows over the record's planes; a
        // warp takes four consecutive records per step (records of a class
        // range are ordered by first plane, so the four mostly share planes)
        const int g = lane >> 3, i = lane & 7;
        const int gbase = lane & ~7;
        for (int m0 = warp * 4; m0 < n_round; m0 += kThreads / 8) {
          const int m = m0 + g;
          const bool valid = m < n_round;
          const int mm = valid ? m : m0;
          const float4 a = stage[mm][0], b = stage[mm][1];
          const uint32_t s = stage_s[mm];
          const int iu_rel = __float_as_int(b.y) - tu * T;
          const int iv_rel = __float_as_int(b.z) - tv * T;
          const int ip = __float_as_int(b.w);
          int pa = max(ip, q0), pb = min(ip + W - 1, q1 - 1);
          if (!valid) pa = pb + 1;
          // kernel values at index i along u, v and w
          float ku = 0.f, kv = 0.f, kw = 0.f;
          if (i < W) {
            ku = es_eval(p.beta, (a.z + (float)i) * inv_half);
            kv = es_eval(p.beta, (a.w + (float)i) * inv_half);
            kw = p.n_planes == 1 ? (i == 0 ? 1.0f : 0.0f)
                                 : es_eval(p.beta, (b.x + (float)i) * inv_half);
          }
          float2 kvj[W];  // the v weights as (w, w) pairs for paired FMAs
#pragma unroll
          for (int j = 0; j < W; ++j) {
            const float k = __shfl_sync(0xffffffffu, kv, gbase + j);
            kvj[j] = make_float2(k, k);
          }
          // the union of the four records' planes; each group reads only its
          // own footprint cells (rows outside every footprint may hold
          // anything in prediction)
          const int qa = __reduce_min_sync(0xffffffffu, pa <= pb ? pa : 0x7fffffff);
          const int qb = __reduce_max_sync(0xffffffffu, pa <= pb ? pb : -0x7fffffff);
          const float2 *col = halo + iv_rel * RS + iu_rel + i;
          float2 s2 = make_float2(0.f, 0.f);
          for (int q = qa; q <= qb; ++q) {
            const int dz = q - ip;
            const float kwq = __shfl_sync(0xffffffffu, kw, gbase + min(max(dz, 0), 7));
            if (q >= pa && q <= pb && i < W) {
              const float2 *c = col + (q - q0) * kPlane;
              float2 cc = make_float2(0.f, 0.f);
#pragma unroll
              for (int j = 0; j < W; ++j) cc = __ffma2_rn(kvj[j], c[j * RS], cc);
              s2 = __ffma2_rn(make_float2(kwq, kwq), cc, s2);
            }
          }
          float sr = s2.x * ku, si = s2.y * ku;
#pragma unroll
          for (int o = 4; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
          }
          // times the conjugate of the record's phase factor (re, im)
          if (i == 0 && pa <= pb)
            atomicAdd(&acc[s], make_float2(fmaf(sr, a.x, si * a.y), fmaf(si, a.x, -sr * a.y)));
        }
      } else {
        // one warp per record (W > 8): lanes own footprint cells
        for (int m = warp; m < n_round; m += kThreads / 32) {
          const uint32_t s = stage_s[m];
          VisRecord v;
          {
            const float4 a = stage[m][0], b = stage[m][1];
            v.re = a.x; v.im = a.y; v.fu = a.z; v.fv = a.w; v.fw = b.x;
            v.iu = __float_as_int(b.y); v.iv = __float_as_int(b.z); v.ip = __float_as_int(b.w);
          }
          const int iu_rel = v.iu - tu * T;
          const int iv_rel = v.iv - tv * T;
          const int pa = max(v.ip, q0), pb = min(v.ip + W - 1, q1 - 1);
          if (pa > pb) continue;  // uniform in the warp
          // kernel weights: lanes [0, W) along u, [W, 2W) along v; along w
          // lanes [2W, 3W) of k1 when 3W <= 32, else lanes [0, W) of k2
          constexpr bool kOneEval = 3 * W <= 32;
          constexpr int kW0 = kOneEval ? 2 * W : 0;
          const int sec = lane < W ? 0 : (lane < 2 * W ? 1 : 2);
          float k1, k2 = 0.f;
          if (kOneEval) {
            const float f1 = (sec == 0 ? v.fu : sec == 1 ? v.fv : v.fw) + (float)(lane - sec * W);
            k1 = lane < 3 * W ? es_eval(p.beta, f1 * inv_half) : 0.f;
            if (p.n_planes == 1 && sec == 2) k1 = lane == 2 * W ? 1.0f : 0.0f;
          } else {
            const float f1 = (sec == 0 ? v.fu : v.fv) + (float)(sec == 0 ? lane : lane - W);
            k1 = lane < 2 * W ? es_eval(p.beta, f1 * inv_half) : 0.f;
            k2 = es_eval(p.beta, (v.fw + (float)lane) * inv_half);
            if (p.n_planes == 1) k2 = lane == 0 ? 1.0f : 0.0f;
          }
          float wgt[kLaneCells];
          int idx[kLaneCells];
  #pragma unroll
          for (int k = 0; k < kLaneCells; ++k) {
            const int c = lane + 32 * k;
            const int i = c % W, j = c / W;
            const float kx = __shfl_sync(0xffffffffu, k1, i);
            const float ky = __shfl_sync(0xffffffffu, k1, W + (j < W ? j : 0));
            // lanes past the footprint read its corner cell with weight 0 (a
            // footprint cell: planes rows outside every footprint are never
            // written in prediction and may hold anything)
            wgt[k] = c < kFoot ? kx * ky : 0.f;
            idx[k] = c < kFoot ? (iv_rel + j) * RS + iu_rel + i : iv_rel * RS + iu_rel;
          }
          float sr = 0.f, si = 0.f;
          for (int q = pa; q <= pb; ++q) {
            const float kw = __shfl_sync(0xffffffffu, kOneEval ? k1 : k2, kW0 + q - v.ip);
            const float2 *pl = halo + (q - q0) * kPlane;
            float pr = 0.f, pi = 0.f;
  #pragma unroll
            for (int k = 0; k < kLaneCells; ++k) {
              const float2 g = pl[idx[k]];
              pr = fmaf(wgt[k], g.x, pr);
              pi = fmaf(wgt[k], g.y, pi);
            }
            sr = fmaf(kw, pr, sr);
            si = fmaf(kw, pi, si);
          }
  #pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
          }
          // times the conjugate of the record's phase factor
          if (lane == 0)
            atomicAdd(&acc[s], make_float2(fmaf(sr, v.re, si * v.im), fmaf(si, v.re, -sr * v.im)));
        }
      }
      __syncthreads();
    }
  }
}

// Zeroes the cells of the gridding units that are split into several items
// (their items add into the planes and into the unit's spill slot); one warp
// per unit.
template <int T, int G>
__global__ void __launch_bounds__(kThreads)
    zero_split_units_kernel(DevPlan p, const uint32_t *__restrict__ item_off, int p_begin,
                            int n_batch, int n_units, const int *__restrict__ slots,
                            float2 *__restrict__ spill, float2 *__restrict__ planes) {
  const int unit = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (unit >= n_units) return;
  if (item_off[unit + 1] - item_off[unit] <= 1) return;
  const int n_tiles = p.ntu * p.ntv;
  const int tile = unit % n_tiles, group = unit / n_tiles;
  const int tu = tile % p.ntu, tv = tile / p.ntu;
  const int q0 = p_begin + group * G;
  const int q1 = min(q0 + G, p_begin + n_batch);
  const size_t plane_elems = (size_t)p.nu * p.nv;
  for (int c = lane; c < (q1 - q0) * T * T; c += 32) {
    const int pq = c / (T * T), rem = c - pq * T * T;
    const int row = rem / T, col = rem - row * T;
    planes[(size_t)(q0 + pq - p_begin) * plane_elems + (size_t)(tv * T + row) * p.nu +
           tu * T + col] = make_float2(0.f, 0.f);
  }
  const int slot = slots[unit];
  if (slot >= 0) {
    const int B = (p.support - 1) * (T + p.support - 1) + (p.support - 1) * T;
    float2 *sp = spill + (size_t)slot * slot_cells(G, B);
    for (int c = lane; c < (q1 - q0) * B; c += 32) sp[c] = make_float2(0.f, 0.f);
    if (lane == 0) sp[G * B] = make_float2(0.f, 0.f);  // the plane mask
  }
}

// Plans the work items of one batch: scanned item offsets (n_units + 1) and
// the item -> unit descriptors, in buffers from `alloc`; for gridding also the
// units' spill slots and the spill buffer.  The numbers of items and slots
// size the launches (one small device-to-host read).
template <int T, int G>
WorkItems plan_items(const DevPlan &p, const uint32_t *off, int p_begin, int n_batch,
                     bool degrid, const ItemAlloc &alloc, cudaStream_t s) {
  WorkItems wi;
  const int n_groups = (n_batch + G - 1) / G;
  wi.n_units = p.ntu * p.ntv * n_groups;
  // [item_off: n_units + 2][counts: n_units + 2][slots: n_units + 2]
  const size_t words = 3 * ((size_t)wi.n_units + 2);
  wi.item_off = (uint32_t *)alloc(0, sizeof(uint32_t) * words);
  uint32_t *counts = wi.item_off + wi.n_units + 2;
  uint32_t *slots = counts + wi.n_units + 2;
  const int warps_per_block = kThreads / 32;
  const unsigned blocks = (unsigned)((wi.n_units + warps_per_block - 1) / warps_per_block);
  grid_plan_kernel<T, G><<<blocks, kThreads, 0, s>>>(p, off, p_begin, n_batch, wi.n_units,
                                                     degrid ? 1 : 0, wi.item_off, counts);
  check_launch("grid_plan_kernel");
  WGPU_CUDA(cudaMemsetAsync(wi.item_off + wi.n_units, 0, sizeof(uint32_t), s));
  uint32_t *tmp = (uint32_t *)alloc(2, sizeof(uint32_t) * exclusive_scan_scratch_words(wi.n_units + 1));
  exclusive_scan_u32_scratch(wi.item_off, wi.n_units + 1, tmp, s);
  if (!degrid) {
    slot_flags_kernel<<<(wi.n_units + 256) / 256, 256, 0, s>>>(counts, wi.n_units, slots);
    check_launch("slot_flags_kernel");
    exclusive_scan_u32_scratch(slots, wi.n_units + 1, tmp, s);
  }
  uint32_t totals[2] = {0, 0};
  WGPU_CUDA(cudaMemcpyAsync(&totals[0], wi.item_off + wi.n_units, sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, s));
  if (!degrid)
    WGPU_CUDA(cudaMemcpyAsync(&totals[1], slots + wi.n_units, sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaStreamSynchronize(s));
  wi.total = totals[0];
  wi.desc = (uint32_t *)alloc(1, sizeof(uint32_t) * ((size_t)wi.total + 1));
  fill_items_kernel<<<(wi.n_units + 255) / 256, 256, 0, s>>>(wi.item_off, counts, wi.n_units,
                                                              wi.desc);
  check_launch("fill_items_kernel");
  if (!degrid) {
    slot_final_kernel<<<(wi.n_units + 255) / 256, 256, 0, s>>>(counts, wi.n_units, (int *)slots);
    check_launch("slot_final_kernel");
    wi.slot = (int *)slots;
    wi.n_slots = (int)totals[1];
    const size_t B = (size_t)spill_cells(T, p.support);
    wi.spill = (float2 *)alloc(3, sizeof(float2) * ((size_t)wi.n_slots * slot_cells(G, (int)B) + 1));
  }
  return wi;
}

template <int T, int G, int W>
void grid_items(const DevPlan &p, const VisRecord *rec, const uint32_t *off, int p_begin,
                int n_batch, const WorkItems &wi, float2 *planes, cudaStream_t s) {
  if (wi.total == 0) return;
  const size_t smem = grid_kernel_smem_bytes<T, G, W>();
  ensure_dynamic_smem((const void *)grid_kernel<T, G, W>, smem);
  int per_sm = 0;
  WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grid_kernel<T, G, W>,
                                                          kThreads, smem));
  const uint32_t blocks = std::min<uint32_t>(wi.total, (uint32_t)(sm_count() * std::max(per_sm, 1)));
  grid_kernel<T, G, W><<<blocks, kThreads, smem, s>>>(p, rec, off, p_begin, n_batch,
                                                      wi.item_off, wi.desc, wi.slot, wi.spill,
                                                      wi.total, planes);
  check_launch("grid_kernel");
}

template <int T, int G, int W>
void degrid_items(const DevPlan &p, const VisRecord *rec, const uint32_t *off, int p_begin,
                  int n_batch, const WorkItems &wi, const float2 *planes, float2 *acc,
                  unsigned *err, cudaStream_t s) {
  if (wi.total == 0) return;
  // a halo row (RS cells, wrapping once at the u edge) must fit in a grid row
  if (p.nu < degrid_row_stride(T + W - 1) || p.nv < T + W - 1)
    throw Error(WGPU_ERR_INVALID, "grid smaller than the degridding halo");
  const size_t smem = degrid_smem_bytes<T, G, W>();
  ensure_dynamic_smem((const void *)degrid_kernel<T, G, W>, smem);
  int per_sm = 0;
  WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, degrid_kernel<T, G, W>,
                                                          kThreads, smem));
  const uint32_t blocks = std::min<uint32_t>(wi.total, (uint32_t)(sm_count() * std::max(per_sm, 1)));
  degrid_kernel<T, G, W><<<blocks, kThreads, smem, s>>>(p, rec, off, p_begin, n_batch,
                                                        wi.item_off, wi.desc, wi.total, planes,
                                                        acc, err);
  check_launch("degrid_kernel");
}

template <int T, int G, int W>
void grid_items_multi(const GridJob *d_jobs, const uint32_t *d_base, int n_jobs, uint32_t total,
                      cudaStream_t s) {
  if (total == 0) return;
  const size_t smem = grid_kernel_smem_bytes<T, G, W>();
  ensure_dynamic_smem((const void *)grid_kernel_multi<T, G, W>, smem);
  int per_sm = 0;
  WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grid_kernel_multi<T, G, W>,
                                                          kThreads, smem));
  const uint32_t blocks = std::min<uint32_t>(total, (uint32_t)(sm_count() * std::max(per_sm, 1)));
  grid_kernel_multi<T, G, W><<<blocks, kThreads, smem, s>>>(d_jobs, d_base, n_jobs, total);
  check_launch("grid_kernel_multi");
}

template <int T, int W = 4>
void grid_multi_dispatch(int support, const GridJob *d_jobs, const uint32_t *d_base, int n_jobs,
                         uint32_t total, cudaStream_t s) {
  if constexpr (W > kMaxSupport) {
    throw Error(WGPU_ERR_INVALID, "kernel support out of range");
  } else {
    if (support == W)
      grid_items_multi<T, grid_group(W), W>(d_jobs, d_base, n_jobs, total, s);
    else
      grid_multi_dispatch<T, W + 1>(support, d_jobs, d_base, n_jobs, total, s);
  }
}

// Dispatch over the kernel support (4..16); the plane group follows W.
template <int T, int W = 4>
void grid_dispatch(int support, const DevPlan &p, const VisRecord *rec, const uint32_t *off,
                   int p_begin, int n_batch, const WorkItems &wi, float2 *planes,
                   cudaStream_t s) {
  if constexpr (W > kMaxSupport) {
    throw Error(WGPU_ERR_INVALID, "kernel support out of range");
  } else {
    if (support == W)
      grid_items<T, grid_group(W), W>(p, rec, off, p_begin, n_batch, wi, planes, s);
    else
      grid_dispatch<T, W + 1>(support, p, rec, off, p_begin, n_batch, wi, planes, s);
  }
}

template <int T, int G, int W = 4>
void degrid_dispatch(int support, const DevPlan &p, const VisRecord *rec, const uint32_t *off,
                     int p_begin, int n_batch, const WorkItems &wi, const float2 *planes,
                     float2 *acc, unsigned *err, cudaStream_t s) {
  if constexpr (W > kMaxSupport || (G > 8 && W > 8)) {
    throw Error(WGPU_ERR_INVALID, "kernel support out of range");
  } else {
    if (support == W)
      degrid_items<T, G, W>(p, rec, off, p_begin, n_batch, wi, planes, acc, err, s);
    else
      degrid_dispatch<T, G, W + 1>(support, p, rec, off, p_begin, n_batch, wi, planes, acc, err,
                                   s);
  }
}

void check_plan(const DevPlan &p) {
  if (p.support < 4 || p.support > kMaxSupport)
    throw Error(WGPU_ERR_INVALID, "kernel support must be 4..16");
  if (p.tile != kTile) throw Error(WGPU_ERR_INVALID, "uv tile must be 16 cells");
}

// w planes per degridding unit: 8 keeps the halo region of a 16x16 tile at
// ~35 KB (W = 8), five blocks per SM.  16 planes read 23% fewer records per
// visibility but fit three blocks per SM (with 128-record rounds), which
// measured 3% slower on the wide-field workload.
constexpr int kDegridPlanes = 8;

}  // namespace

int grid_plane_group() { return kGridPlanes; }

WorkItems plan_grid_items(const DevPlan &p, const uint32_t *off, int p_begin, int n_batch,
                          const ItemAlloc &alloc, cudaStream_t s) {
  check_plan(p);
  if (p.support <= 8)
    return plan_items<kTile, grid_group(8)>(p, off, p_begin, n_batch, false, alloc, s);
  return plan_items<kTile, grid_group(16)>(p, off, p_begin, n_batch, false, alloc, s);
}

WorkItems plan_degrid_items(const DevPlan &p, const uint32_t *off, int p_begin, int n_batch,
                            const ItemAlloc &alloc, cudaStream_t s) {
  check_plan(p);
  return plan_items<kTile, kDegridPlanes>(p, off, p_begin, n_batch, true, alloc, s);
}

void launch_zero_split_units(const DevPlan &p, const WorkItems &wi, int p_begin, int n_batch,
                             float2 *planes, cudaStream_t s) {
  const int warps_per_block = kThreads / 32;
  const unsigned blocks = (unsigned)((wi.n_units + warps_per_block - 1) / warps_per_block);
  if (p.support <= 8)
    zero_split_units_kernel<kTile, grid_group(8)><<<blocks, kThreads, 0, s>>>(
        p, wi.item_off, p_begin, n_batch, wi.n_units, wi.slot, wi.spill, planes);
  else
    zero_split_units_kernel<kTile, grid_group(16)><<<blocks, kThreads, 0, s>>>(
        p, wi.item_off, p_begin, n_batch, wi.n_units, wi.slot, wi.spill, planes);
  check_launch("zero_split_units_kernel");
}

size_t grid_spill_elems(const DevPlan &p, const WorkItems &wi) {
  const int G = p.support <= 8 ? grid_group(8) : grid_group(16);
  return (size_t)wi.n_slots * slot_cells(G, spill_cells(kTile, p.support));
}

void launch_spill_fixup(const DevPlan &p, const WorkItems &wi, int p_begin, int n_batch,
                        float2 *planes, cudaStream_t s) {
  if (wi.n_slots == 0 || p.support < 2) return;
  const int G = p.support <= 8 ? grid_group(8) : grid_group(16);
  const unsigned blocks = (unsigned)std::min<int64_t>(wi.n_units, (int64_t)sm_count() * 8);
  spill_fixup_kernel<<<blocks, kThreads, 0, s>>>(p, G, p_begin, n_batch, wi.n_units, wi.slot,
                                                  wi.spill, planes);
  check_launch("spill_fixup_kernel");
}

void launch_grid_items(const DevPlan &p, const VisRecord *rec, const uint32_t *off, int p_begin,
                       int n_batch, const WorkItems &wi, float2 *planes, cudaStream_t s) {
  check_plan(p);
  grid_dispatch<kTile>(p.support, p, rec, off, p_begin, n_batch, wi, planes, s);
  launch_spill_fixup(p, wi, p_begin, n_batch, planes, s);
}

template <int T, int W = 4>
void grid_multi_prepare(int support) {
  if constexpr (W <= kMaxSupport) {
    if (support == W)
      ensure_dynamic_smem((const void *)grid_kernel_multi<T, grid_group(W), W>,
                          grid_kernel_smem_bytes<T, grid_group(W), W>());
    else
      grid_multi_prepare<T, W + 1>(support);
  }
}

void prepare_grid_items_multi(int support) { grid_multi_prepare<kTile>(support); }

void launch_grid_items_multi(int support, const GridJob *d_jobs, const uint32_t *d_base,
                             int n_jobs, uint32_t total, cudaStream_t s) {
  if (support < 4 || support > kMaxSupport)
    throw Error(WGPU_ERR_INVALID, "kernel support must be 4..16");
  grid_multi_dispatch<kTile>(support, d_jobs, d_base, n_jobs, total, s);
}

void launch_degrid_items(const DevPlan &p, const VisRecord *rec, const uint32_t *off,
                         int p_begin, int n_batch, const WorkItems &wi, const float2 *planes,
                         float2 *acc, unsigned *err, cudaStream_t s) {
  check_plan(p);
  degrid_dispatch<kTile, kDegridPlanes>(p.support, p, rec, off, p_begin, n_batch, wi, planes, acc,
                                        err, s);
}

static ItemAlloc arena_alloc(DeviceArena &arena) {
  return [&arena](int which, size_t bytes) -> void * {
    const int slot = which == 0   ? kSlotItems
                     : which == 1 ? kSlotItemDesc
                     : which == 2 ? kSlotScanTmp
                                  : kSlotSpill;
    return arena.get(slot, bytes);
  };
}

void launch_grid(DeviceArena &arena, const DevPlan &p, const VisRecord *rec,
                 const uint32_t *off, int p_begin, int n_batch, float2 *planes,
                 cudaStream_t s) {
  const WorkItems wi = plan_grid_items(p, off, p_begin, n_batch, arena_alloc(arena), s);
  launch_zero_split_units(p, wi, p_begin, n_batch, planes, s);
  launch_grid_items(p, rec, off, p_begin, n_batch, wi, planes, s);
}

void launch_degrid(DeviceArena &arena, const DevPlan &p, const VisRecord *rec,
                   const uint32_t *off, int p_begin, int n_batch, const float2 *planes,
                   float2 *acc, unsigned *err, cudaStream_t s) {
  const WorkItems wi = plan_degrid_items(p, off, p_begin, n_batch, arena_alloc(arena), s);
  launch_degrid_items(p, rec, off, p_begin, n_batch, wi, planes, acc, err, s);
}

}  // namespace wgpu
