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
// Gridding item: a block keeps the unit's cells in shared memory; each warp
// owns two rows of every plane and adds the footprints of the staged records
// with plain read-add-writes; the tile is written to HBM once per item (a
// unit split into several items adds into cells zeroed beforehand).  One
// launch can also serve many jobs (facets x channel groups), each with its own
// plan, records and planes (grid_kernel_multi).
//
// Degridding item: loads its tile plus a (W-1)-cell halo of G planes into
// shared memory and gathers, for each visibility of its slice of the own
// bucket, the W x W x (planes in the group) weighted sum, added to the
// per-visibility accumulator.
#include <algorithm>

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
  // planes is null when the items are planned ahead of the gridding (bound
  // sets); zero_split_units_kernel then clears these cells before each pass.
  if (!degrid && planes != nullptr && n_items > 1) {
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

// Shared-memory layout of the gridding kernel: the tile's float2 cells
// [G][T][T], then the staged round: five meta arrays [5][kGridRound] (re, im,
// u and v corner relative to the tile, first plane relative to the group) and
// the kernel values [kGridRound][kw] with kw = 3W rounded up to an odd count
// (kx[W], ky[W], kz[W] per record; the odd stride keeps the stores of a warp
// on distinct banks).
constexpr int kGridRound = 32;  // records staged per round (eight threads stage each)
__host__ __device__ constexpr int grid_weight_stride(int W) { return (3 * W) | 1; }
template <int T, int G, int W>
constexpr size_t grid_smem_bytes() {
  return sizeof(float2) * G * T * T +
         sizeof(float) * kGridRound * (5 + grid_weight_stride(W));
}

// Gridding of one plane batch.  The block owns one unit (a T x T tile over G
// planes) per work item and keeps its cells in shared memory.  Warp k owns
// rows 2k and 2k+1 of every plane, so a cell is only ever updated by one warp:
// plain load-multiply-add-store, no atomics.  Each round stages up to
// kGridRound visibility reads with their kernel values (evaluated once per
// read); every warp scans the round and adds the part of each footprint that
// falls on its two rows: lanes cover (footprint column, row of the pair,
// plane parity) and step through the footprint's planes.  Columns are
// XOR-swizzled by row parity so that the 64-bit accesses of a half-warp (two
// rows x eight columns) fall on distinct banks.  A work item holds at most
// kItemVis reads, which bounds the FP32 accumulation chain of every cell; the
// tile is flushed to HBM once at the item's end.

// Shared memory of the gridding kernels (see grid_smem_bytes).
struct GridSmem {
  float2 *cells;
  float *m_re, *m_im;
  int *m_iu, *m_iv, *m_ip;
  float *wts;
  uint32_t *rs0, *rcum;
};

template <int T, int G, int W>
__device__ __forceinline__ GridSmem grid_smem(float4 *smem4, uint32_t *rs0, uint32_t *rcum) {
  constexpr int kCells = T * T;
  GridSmem sm;
  sm.cells = reinterpret_cast<float2 *>(smem4);  // [G][T][T], swizzled columns
  sm.m_re = reinterpret_cast<float *>(sm.cells + G * kCells);
  sm.m_im = sm.m_re + kGridRound;
  sm.m_iu = reinterpret_cast<int *>(sm.m_im + kGridRound);
  sm.m_iv = sm.m_iu + kGridRound;
  sm.m_ip = sm.m_iv + kGridRound;
  sm.wts = reinterpret_cast<float *>(sm.m_ip + kGridRound);  // [kGridRound][kWS]
  sm.rs0 = rs0;
  sm.rcum = rcum;
  return sm;
}

// One work item (descriptor d, item index `item` of its plane batch).  The
// tile cells are zero on entry and on return; ends with a block barrier
// unless the unit has no visibilities.
template <int T, int G, int W>
__device__ __forceinline__ void grid_item(const DevPlan &p, const VisRecord *__restrict__ rec,
                                          const uint32_t *__restrict__ off, int p_begin,
                                          int n_batch, const uint32_t *__restrict__ item_off,
                                          uint32_t d, uint32_t item,
                                          float2 *__restrict__ planes, const GridSmem &sm) {
  constexpr int kCols = W <= 8 ? 8 : 16;            // lanes across footprint columns
  constexpr int kPlaneLanes = 32 / (2 * kCols);     // 2 (W <= 8) or 1
  constexpr int kSteps = (W + kPlaneLanes - 1) / kPlaneLanes;
  constexpr int kWS = grid_weight_stride(W);
  constexpr int kCells = T * T;
  float2 *cells = sm.cells;
  float *m_re = sm.m_re, *m_im = sm.m_im, *wts = sm.wts;
  int *m_iu = sm.m_iu, *m_iv = sm.m_iv, *m_ip = sm.m_ip;
  uint32_t *rs0 = sm.rs0, *rcum = sm.rcum;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ci = lane % kCols;              // footprint column offset
  const int row = 2 * warp + ((lane / kCols) & 1);
  const int pj = lane / (2 * kCols);        // plane parity (W <= 8)
  const int swz = (row & 1) << 3;
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
    // no visibility reaches this unit: its cells are zero
    for (int c = threadIdx.x; c < nq * kCells; c += kThreads) {
      const int pq = c / kCells, rem = c - pq * kCells;
      const int rr = rem / T, cc = rem - rr * T;
      planes[(size_t)(q0 + pq - p_begin) * plane_elems + (size_t)(tv * T + rr) * p.nu +
             tu * T + cc] = make_float2(0.f, 0.f);
    }
    return;
  }
  const uint32_t first = __ldg(item_off + unit);
  const uint32_t n_items = __ldg(item_off + unit + 1) - first;
  if (threadIdx.x < 9) {
    uint32_t a, b;
    unit_range(p, off, tile, q0, q1, threadIdx.x, &a, &b);
    rs0[threadIdx.x] = a;
    rcum[threadIdx.x + 1] = b - a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    rcum[0] = 0;
    for (int r = 0; r < 9; ++r) rcum[r + 1] += rcum[r];
  }
  __syncthreads();
  const uint32_t lo = (item - first) * kItemVis;
  const uint32_t hi = min(lo + kItemVis, rcum[9]);

  for (uint32_t rb = lo; rb < hi; rb += kGridRound) {
    // stage: eight threads share read t; roles 0-5 evaluate half of kx, ky
    // or kz each, role 6 writes the meta data
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
        if (role < 6) {
          const int dim = role >> 1, k0 = (role & 1) * kHalf;
          const float f = dim == 0 ? v.fu : (dim == 1 ? v.fv : v.fw);
#pragma unroll
          for (int kk = 0; kk < kHalf; ++kk) {
            const int k = k0 + kk;
            if (k < W)
              w[dim * W + k] = (dim == 2 && p.n_planes == 1)
                                   ? (k == 0 ? 1.0f : 0.0f)
                                   : es_eval(p.beta, (f + (float)k) * inv_half);
          }
        } else {
          int iu_rel = v.iu - tu * T;
          if (iu_rel >= T) iu_rel -= p.nu;
          int iv_rel = v.iv - tv * T;
          if (iv_rel >= T) iv_rel -= p.nv;
          m_re[t] = v.re;
          m_im[t] = v.im;
          m_iu[t] = iu_rel;
          m_iv[t] = iv_rel;
          m_ip[t] = v.ip - q0;
        }
      }
    }
    __syncthreads();
    const int n_round = (int)min((uint32_t)kGridRound, hi - rb);
    for (int m = 0; m < n_round; ++m) {
      const int ivr = m_iv[m];
      if (ivr > 2 * warp + 1 || ivr + W <= 2 * warp) continue;  // uniform in the warp
      const int col = m_iu[m] + ci;
      const int dv = row - ivr;
      if (ci < W && col >= 0 && col < T && dv >= 0 && dv < W) {
        const float *w = wts + m * kWS;
        const int ipr = m_ip[m];
        const float re = m_re[m], im = m_im[m];
        const float wuv = w[ci] * w[W + dv];
        float2 *cb = cells + row * T + (col ^ swz);
#pragma unroll
        for (int s = 0; s < kSteps; ++s) {
          const int dz = s * kPlaneLanes + pj;
          const int q = ipr + dz;
          if (dz < W && q >= 0 && q < nq) {
            const float t = wuv * w[2 * W + dz];
            float2 c = cb[q * kCells];
            c.x = fmaf(t, re, c.x);
            c.y = fmaf(t, im, c.y);
            cb[q * kCells] = c;
          }
        }
      }
      __syncwarp();  // the next read's lanes may update the same cells
    }
    __syncthreads();
  }
  // flush the tile (a split unit adds into cells zeroed beforehand)
  for (int c = threadIdx.x; c < G * kCells; c += kThreads) {
    const int pq = c / kCells, rem = c - pq * kCells;
    const int rr = rem / T, cc = rem - rr * T;
    float2 *src = cells + pq * kCells + rr * T + (cc ^ ((rr & 1) << 3));
    const float2 val = *src;
    *src = make_float2(0.f, 0.f);
    if (pq < nq) {
      float2 *dst = planes + (size_t)(q0 + pq - p_begin) * plane_elems +
                    (size_t)(tv * T + rr) * p.nu + tu * T + cc;
      if (n_items == 1)
        *dst = val;
      else
        atomicAdd(dst, val);
    }
  }
  __syncthreads();
}

template <int T, int G, int W>
__global__ void __launch_bounds__(kThreads)
    grid_kernel(DevPlan p, const VisRecord *__restrict__ rec,
                const uint32_t *__restrict__ off, int p_begin, int n_batch,
                const uint32_t *__restrict__ item_off, const uint32_t *__restrict__ desc,
                uint32_t total, float2 *__restrict__ planes) {
  static_assert(T == 16 && kThreads == 256, "eight warps own two tile rows each");
  extern __shared__ float4 smem4[];
  __shared__ uint32_t rs0[9], rcum[10];
  const GridSmem sm = grid_smem<T, G, W>(smem4, rs0, rcum);
  for (int c = threadIdx.x; c < G * T * T; c += kThreads) sm.cells[c] = make_float2(0.f, 0.f);
  __syncthreads();
  for (uint32_t item = blockIdx.x; item < total; item += gridDim.x)
    grid_item<T, G, W>(p, rec, off, p_begin, n_batch, item_off, __ldg(desc + item), item, planes,
                       sm);
}

// Several gridding jobs (facets x channel groups, each with its own plan,
// records and planes but the same kernel support) in one persistent launch:
// item i belongs to the job j with job_base[j] <= i < job_base[j + 1]; the
// block keeps the current job's description in shared memory.
template <int T, int G, int W>
__global__ void __launch_bounds__(kThreads)
    grid_kernel_multi(const GridJob *__restrict__ jobs, const uint32_t *__restrict__ job_base,
                      int n_jobs, uint32_t total) {
  static_assert(T == 16 && kThreads == 256, "eight warps own two tile rows each");
  static_assert(sizeof(GridJob) % 8 == 0, "job copied in 8-byte words");
  extern __shared__ float4 smem4[];
  __shared__ uint32_t rs0[9], rcum[10];
  __shared__ GridJob job;
  const GridSmem sm = grid_smem<T, G, W>(smem4, rs0, rcum);
  for (int c = threadIdx.x; c < G * T * T; c += kThreads) sm.cells[c] = make_float2(0.f, 0.f);
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
    grid_item<T, G, W>(job.p, job.rec, job.off, job.p_begin, job.n_batch, job.item_off,
                       __ldg(job.desc + local), local, job.planes, sm);
  }
}

// Degridding of one plane batch, one warp per visibility: the block loads
// its unit's halo region (the tile plus W - 1 cells, G planes) into shared
// memory as float2 cells with a row stride of T + W rounded to 8 mod 16 (a
// half-warp's two rows x eight columns then fall on distinct bank pairs);
// lanes own footprint cells, accumulate their cells over the planes of the
// group, and a warp-level shuffle reduction forms the sum.
__host__ __device__ constexpr int degrid_row_stride(int R) { return (R + 7) / 16 * 16 + 8; }
template <int T, int G, int W>
constexpr size_t degrid_smem_bytes() {
  return sizeof(float2) * G * (T + W - 1) * degrid_row_stride(T + W - 1);
}

template <int T, int G, int W>
__global__ void __launch_bounds__(kThreads)
    degrid_kernel(DevPlan p, const VisRecord *__restrict__ rec,
                  const uint32_t *__restrict__ off, int p_begin, int n_batch,
                  const uint32_t *__restrict__ item_off, const uint32_t *__restrict__ desc,
                  uint32_t total, const float2 *__restrict__ planes,
                  float2 *__restrict__ acc) {
  constexpr int R = T + W - 1;
  constexpr int RS = degrid_row_stride(R);
  constexpr int kPlane = R * RS;
  constexpr int kFoot = W * W;
  constexpr int kLaneCells = (kFoot + 31) / 32;
  extern __shared__ float2 halo[];  // [G][R][RS]
  __shared__ uint32_t rs0[4], rcum[5];
  __shared__ float4 stage[kThreads][2];
  __shared__ uint32_t stage_s[kThreads];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float inv_half = 2.0f / (float)W;
  const int n_tiles = p.ntu * p.ntv;
  const size_t plane_elems = (size_t)p.nu * p.nv;

  for (uint32_t item = blockIdx.x; item < total; item += gridDim.x) {
    const int unit = (int)(__ldg(desc + item) & 0x7fffffffu);
    const int tile = unit % n_tiles, group = unit / n_tiles;
    const int tu = tile % p.ntu, tv = tile / p.ntu;
    const int q0 = p_begin + group * G;
    const int q1 = min(q0 + G, p_begin + n_batch);
    const uint32_t lo = (item - __ldg(item_off + unit)) * kItemVis;

    const int nq = q1 - q0;
    for (int idx = threadIdx.x; idx < nq * R * R; idx += blockDim.x) {
      const int pq = idx / (R * R), rem = idx - pq * R * R;
      const int r = rem / R, c = rem - r * R;
      int gv = tv * T + r;
      if (gv >= p.nv) gv -= p.nv;
      int gu = tu * T + c;
      if (gu >= p.nu) gu -= p.nu;
      halo[pq * kPlane + r * RS + c] =
          __ldg(planes + (size_t)(q0 + pq - p_begin) * plane_elems + (size_t)gv * p.nu + gu);
    }
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
    const uint32_t hi = min(lo + kItemVis, rcum[4]);

    for (uint32_t rb = lo; rb < hi; rb += kThreads) {
      {
        const uint32_t pos = rb + threadIdx.x;
        if (pos < hi) {
          int r = 0;
          while (pos >= rcum[r + 1]) ++r;
          const uint32_t s = rs0[r] + (pos - rcum[r]);
          const float4 *src = reinterpret_cast<const float4 *>(rec + s);
          stage[threadIdx.x][0] = __ldg(src);
          stage[threadIdx.x][1] = __ldg(src + 1);
          stage_s[threadIdx.x] = s;
        }
      }
      __syncthreads();
      const int n_round = (int)min((uint32_t)kThreads, hi - rb);
      for (int m = warp * 32; m < min(n_round, warp * 32 + 32); ++m) {
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
        const bool lx = lane < W;
        const float f1 = (lx ? v.fu : v.fv) + (float)(lx ? lane : lane - W);
        float k1 = es_eval(p.beta, f1 * inv_half);
        k1 = lane < 2 * W ? k1 : 0.f;
        float k2 = es_eval(p.beta, (v.fw + (float)lane) * inv_half);
        if (p.n_planes == 1) k2 = lane == 0 ? 1.0f : 0.0f;
        float wgt[kLaneCells];
        int idx[kLaneCells];
#pragma unroll
        for (int k = 0; k < kLaneCells; ++k) {
          const int c = lane + 32 * k;
          const int i = c % W, j = c / W;
          const float kx = __shfl_sync(0xffffffffu, k1, i);
          const float ky = __shfl_sync(0xffffffffu, k1, W + (j < W ? j : 0));
          wgt[k] = c < kFoot ? kx * ky : 0.f;
          idx[k] = c < kFoot ? (iv_rel + j) * RS + iu_rel + i : 0;
        }
        float sr = 0.f, si = 0.f;
        for (int q = pa; q <= pb; ++q) {
          const float kw = __shfl_sync(0xffffffffu, k2, q - v.ip);
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
        if (lane == 0) atomicAdd(&acc[s], make_float2(sr, si));
      }
      __syncthreads();
    }
  }
}

int sm_count() {
  // initialised once, thread-safely (gridders run on several host threads)
  static const int n = [] {
    int dev = 0, v = 0;
    WGPU_CUDA(cudaGetDevice(&dev));
    WGPU_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    return v;
  }();
  return n;
}

// Zeroes the cells of the gridding units that are split into several items
// (their items add into the planes); one warp per unit.
template <int T, int G>
__global__ void __launch_bounds__(kThreads)
    zero_split_units_kernel(DevPlan p, const uint32_t *__restrict__ item_off, int p_begin,
                            int n_batch, int n_units, float2 *__restrict__ planes) {
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
}

// Plans the work items of one batch: scanned item offsets (n_units + 1) and
// the item -> unit descriptors, in buffers from `alloc`.  The number of items
// sizes the launch (one small device-to-host read).  With `planes` the split
// gridding units are zeroed as well.
template <int T, int G>
WorkItems plan_items(const DevPlan &p, const uint32_t *off, int p_begin, int n_batch,
                     bool degrid, float2 *planes, const ItemAlloc &alloc, cudaStream_t s) {
  WorkItems wi;
  const int n_groups = (n_batch + G - 1) / G;
  wi.n_units = p.ntu * p.ntv * n_groups;
  wi.item_off = (uint32_t *)alloc(0, sizeof(uint32_t) * (2 * (size_t)wi.n_units + 4));
  uint32_t *counts = wi.item_off + wi.n_units + 2;
  const int warps_per_block = kThreads / 32;
  const unsigned blocks = (unsigned)((wi.n_units + warps_per_block - 1) / warps_per_block);
  grid_plan_kernel<T, G><<<blocks, kThreads, 0, s>>>(p, off, p_begin, n_batch, wi.n_units,
                                                     degrid ? 1 : 0, wi.item_off, counts,
                                                     planes);
  check_launch("grid_plan_kernel");
  WGPU_CUDA(cudaMemsetAsync(wi.item_off + wi.n_units, 0, sizeof(uint32_t), s));
  uint32_t *tmp = (uint32_t *)alloc(2, sizeof(uint32_t) * exclusive_scan_scratch_words(wi.n_units + 1));
  exclusive_scan_u32_scratch(wi.item_off, wi.n_units + 1, tmp, s);
  uint32_t total = 0;
  WGPU_CUDA(cudaMemcpyAsync(&total, wi.item_off + wi.n_units, sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaStreamSynchronize(s));
  wi.total = total;
  wi.desc = (uint32_t *)alloc(1, sizeof(uint32_t) * ((size_t)total + 1));
  fill_items_kernel<<<(wi.n_units + 255) / 256, 256, 0, s>>>(wi.item_off, counts, wi.n_units,
                                                              wi.desc);
  check_launch("fill_items_kernel");
  return wi;
}

template <int T, int G, int W>
void grid_items(const DevPlan &p, const VisRecord *rec, const uint32_t *off, int p_begin,
                int n_batch, const WorkItems &wi, float2 *planes, cudaStream_t s) {
  if (wi.total == 0) return;
  const size_t smem = grid_smem_bytes<T, G, W>();
  ensure_dynamic_smem((const void *)grid_kernel<T, G, W>, smem);
  int per_sm = 0;
  WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grid_kernel<T, G, W>,
                                                          kThreads, smem));
  const uint32_t blocks = std::min<uint32_t>(wi.total, (uint32_t)(sm_count() * std::max(per_sm, 1)));
  grid_kernel<T, G, W><<<blocks, kThreads, smem, s>>>(p, rec, off, p_begin, n_batch,
                                                      wi.item_off, wi.desc, wi.total, planes);
  check_launch("grid_kernel");
}

template <int T, int G, int W>
void degrid_items(const DevPlan &p, const VisRecord *rec, const uint32_t *off, int p_begin,
                  int n_batch, const WorkItems &wi, const float2 *planes, float2 *acc,
                  cudaStream_t s) {
  if (wi.total == 0) return;
  const size_t smem = degrid_smem_bytes<T, G, W>();
  ensure_dynamic_smem((const void *)degrid_kernel<T, G, W>, smem);
  int per_sm = 0;
  WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, degrid_kernel<T, G, W>,
                                                          kThreads, smem));
  const uint32_t blocks = std::min<uint32_t>(wi.total, (uint32_t)(sm_count() * std::max(per_sm, 1)));
  degrid_kernel<T, G, W><<<blocks, kThreads, smem, s>>>(p, rec, off, p_begin, n_batch,
                                                        wi.item_off, wi.desc, wi.total, planes,
                                                        acc);
  check_launch("degrid_kernel");
}

template <int T, int G, int W>
void grid_items_multi(const GridJob *d_jobs, const uint32_t *d_base, int n_jobs, uint32_t total,
                      cudaStream_t s) {
  if (total == 0) return;
  const size_t smem = grid_smem_bytes<T, G, W>();
  ensure_dynamic_smem((const void *)grid_kernel_multi<T, G, W>, smem);
  int per_sm = 0;
  WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grid_kernel_multi<T, G, W>,
                                                          kThreads, smem));
  const uint32_t blocks = std::min<uint32_t>(total, (uint32_t)(sm_count() * std::max(per_sm, 1)));
  grid_kernel_multi<T, G, W><<<blocks, kThreads, smem, s>>>(d_jobs, d_base, n_jobs, total);
  check_launch("grid_kernel_multi");
}

template <int T, int G, int W = 4>
void grid_multi_dispatch(int support, const GridJob *d_jobs, const uint32_t *d_base, int n_jobs,
                         uint32_t total, cudaStream_t s) {
  if constexpr (W > kMaxSupport) {
    throw Error(WGPU_ERR_INVALID, "kernel support out of range");
  } else {
    if (support == W)
      grid_items_multi<T, G, W>(d_jobs, d_base, n_jobs, total, s);
    else
      grid_multi_dispatch<T, G, W + 1>(support, d_jobs, d_base, n_jobs, total, s);
  }
}

// Dispatch over the kernel support (4..16).
template <int T, int G, int W = 4>
void grid_dispatch(int support, const DevPlan &p, const VisRecord *rec, const uint32_t *off,
                   int p_begin, int n_batch, const WorkItems &wi, float2 *planes,
                   cudaStream_t s) {
  if constexpr (W > kMaxSupport) {
    throw Error(WGPU_ERR_INVALID, "kernel support out of range");
  } else {
    if (support == W)
      grid_items<T, G, W>(p, rec, off, p_begin, n_batch, wi, planes, s);
    else
      grid_dispatch<T, G, W + 1>(support, p, rec, off, p_begin, n_batch, wi, planes, s);
  }
}

template <int T, int G, int W = 4>
void degrid_dispatch(int support, const DevPlan &p, const VisRecord *rec, const uint32_t *off,
                     int p_begin, int n_batch, const WorkItems &wi, const float2 *planes,
                     float2 *acc, cudaStream_t s) {
  if constexpr (W > kMaxSupport || (G > 8 && W > 8)) {
    throw Error(WGPU_ERR_INVALID, "kernel support out of range");
  } else {
    if (support == W)
      degrid_items<T, G, W>(p, rec, off, p_begin, n_batch, wi, planes, acc, s);
    else
      degrid_dispatch<T, G, W + 1>(support, p, rec, off, p_begin, n_batch, wi, planes, acc, s);
  }
}

void check_plan(const DevPlan &p) {
  if (p.support < 4 || p.support > kMaxSupport)
    throw Error(WGPU_ERR_INVALID, "kernel support must be 4..16");
  if (p.tile != kTile) throw Error(WGPU_ERR_INVALID, "uv tile must be 16 cells");
}

// w planes per degridding unit: 8 keeps the halo region of a 16x16 tile at
// ~35 KB (W = 8), five blocks per SM; 16 planes halve the record reads but
// allow only two blocks per SM, which measured 1.3x slower.
constexpr int kDegridPlanes = 8;

}  // namespace

int grid_plane_group() { return kGridPlanes; }

WorkItems plan_grid_items(const DevPlan &p, const uint32_t *off, int p_begin, int n_batch,
                          float2 *planes, const ItemAlloc &alloc, cudaStream_t s) {
  check_plan(p);
  return plan_items<kTile, kGridPlanes>(p, off, p_begin, n_batch, false, planes, alloc, s);
}

WorkItems plan_degrid_items(const DevPlan &p, const uint32_t *off, int p_begin, int n_batch,
                            const ItemAlloc &alloc, cudaStream_t s) {
  check_plan(p);
  return plan_items<kTile, kDegridPlanes>(p, off, p_begin, n_batch, true, nullptr, alloc, s);
}

void launch_zero_split_units(const DevPlan &p, const WorkItems &wi, int p_begin, int n_batch,
                             float2 *planes, cudaStream_t s) {
  const int warps_per_block = kThreads / 32;
  const unsigned blocks = (unsigned)((wi.n_units + warps_per_block - 1) / warps_per_block);
  zero_split_units_kernel<kTile, kGridPlanes><<<blocks, kThreads, 0, s>>>(
      p, wi.item_off, p_begin, n_batch, wi.n_units, planes);
  check_launch("zero_split_units_kernel");
}

void launch_grid_items(const DevPlan &p, const VisRecord *rec, const uint32_t *off, int p_begin,
                       int n_batch, const WorkItems &wi, float2 *planes, cudaStream_t s) {
  check_plan(p);
  grid_dispatch<kTile, kGridPlanes>(p.support, p, rec, off, p_begin, n_batch, wi, planes, s);
}

template <int T, int G, int W = 4>
void grid_multi_prepare(int support) {
  if constexpr (W <= kMaxSupport) {
    if (support == W)
      ensure_dynamic_smem((const void *)grid_kernel_multi<T, G, W>, grid_smem_bytes<T, G, W>());
    else
      grid_multi_prepare<T, G, W + 1>(support);
  }
}

void prepare_grid_items_multi(int support) {
  grid_multi_prepare<kTile, kGridPlanes>(support);
}

void launch_grid_items_multi(int support, const GridJob *d_jobs, const uint32_t *d_base,
                             int n_jobs, uint32_t total, cudaStream_t s) {
  if (support < 4 || support > kMaxSupport)
    throw Error(WGPU_ERR_INVALID, "kernel support must be 4..16");
  grid_multi_dispatch<kTile, kGridPlanes>(support, d_jobs, d_base, n_jobs, total, s);
}

void launch_degrid_items(const DevPlan &p, const VisRecord *rec, const uint32_t *off,
                         int p_begin, int n_batch, const WorkItems &wi, const float2 *planes,
                         float2 *acc, cudaStream_t s) {
  check_plan(p);
  degrid_dispatch<kTile, kDegridPlanes>(p.support, p, rec, off, p_begin, n_batch, wi, planes, acc,
                                        s);
}

static ItemAlloc arena_alloc(DeviceArena &arena) {
  return [&arena](int which, size_t bytes) -> void * {
    const int slot = which == 0 ? kSlotItems : which == 1 ? kSlotItemDesc : kSlotScanTmp;
    return arena.get(slot, bytes);
  };
}

void launch_grid(DeviceArena &arena, const DevPlan &p, const VisRecord *rec,
                 const uint32_t *off, int p_begin, int n_batch, float2 *planes,
                 cudaStream_t s) {
  const WorkItems wi = plan_grid_items(p, off, p_begin, n_batch, planes, arena_alloc(arena), s);
  launch_grid_items(p, rec, off, p_begin, n_batch, wi, planes, s);
}

void launch_degrid(DeviceArena &arena, const DevPlan &p, const VisRecord *rec,
                   const uint32_t *off, int p_begin, int n_batch, const float2 *planes,
                   float2 *acc, cudaStream_t s) {
  const WorkItems wi = plan_degrid_items(p, off, p_begin, n_batch, arena_alloc(arena), s);
  launch_degrid_items(p, rec, off, p_begin, n_batch, wi, planes, acc, s);
}

}  // namespace wgpu
