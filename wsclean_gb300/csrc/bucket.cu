// K1: visibility bucketing.
//
// Every visibility (row, chan) gets the corner of its W x W x W footprint on
// the oversampled (u, v, w-plane) grid, computed in FP64 from uvw x frequency,
// and a key = (uv tile, first w plane).  A stable LSD radix sort orders the
// visibilities by key and, within a key, by the footprint corner inside the
// tile (its first pass sorts by the corner byte), so that the samples sharing
// an exact footprint corner are consecutive; the bucket offsets come from a
// histogram of the sorted keys and an exclusive scan; finally one 32-byte record per
// visibility is written in sorted order, carrying the visibility times its
// shift phase (inversion) or the phase factor itself (prediction).
//
// The footprint arithmetic uses explicitly rounded operations (__dmul_rn,
// __dsub_rn, never contracted into FMAs) so that the integer corners, the
// float fractions, the keys and the permutation are bit-identical to the CPU
// bucketing reference in oracle/wgpu_oracle.c.
#include <cub/cub.cuh>

#include <mutex>

#include "record_ff.cuh"
#include "wgpu_internal.h"

namespace wgpu {

namespace {

constexpr int kThreads = 256;
// channel counts for which the w extent runs one warp per row
constexpr int64_t kExtentRowsMinChan = 16, kExtentRowsMaxChan = 2048;

struct ChannelScale {
  double su, sv, sw;  // U = uvw_u * su (cells), V = uvw_v * sv, w = uvw_w * sw
  float fsu, fsv, fsw;  // the same rounded to float (FP32 footprint tests)
  float lsu, lsv, lsw;  // the rests rounded to float (float-float records)
};

__global__ void channel_scales_kernel(const double *freq, int64_t n_chan,
                                      double gu, double gv,
                                      ChannelScale *out) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_chan) return;
  const double fl = __ddiv_rn(freq[c], kSpeedOfLight);
  out[c].su = __dmul_rn(fl, gu);
  out[c].sv = __dmul_rn(fl, gv);
  out[c].sw = fl;
  out[c].fsu = __double2float_rn(out[c].su);
  out[c].fsv = __double2float_rn(out[c].sv);
  out[c].fsw = __double2float_rn(fl);
  out[c].lsu = __double2float_rn(__dsub_rn(out[c].su, (double)out[c].fsu));
  out[c].lsv = __double2float_rn(__dsub_rn(out[c].sv, (double)out[c].fsv));
  out[c].lsw = __double2float_rn(__dsub_rn(fl, (double)out[c].fsw));
}

// uvw rows rounded to float (FP32 footprint tests), one float4 per row, and
// the rests rounded to float (float-float records), one float4 per row.
__global__ void uvw_float_kernel(const double *__restrict__ uvw, int64_t n_rows,
                                 float4 *__restrict__ out, float4 *__restrict__ out_lo) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  const double u = uvw[3 * r], v = uvw[3 * r + 1], w = uvw[3 * r + 2];
  const float fu = __double2float_rn(u), fv = __double2float_rn(v), fw = __double2float_rn(w);
  out[r] = make_float4(fu, fv, fw, 0.f);
  out_lo[r] = make_float4(__double2float_rn(__dsub_rn(u, (double)fu)),
                          __double2float_rn(__dsub_rn(v, (double)fv)),
                          __double2float_rn(__dsub_rn(w, (double)fw)), 0.f);
}

// The float row of sample row r: from the table when there is one.
__device__ __forceinline__ float4 row_float(const float4 *uvwf, const double *uvw, int64_t r) {
  if (uvwf) return __ldg(uvwf + r);
  return make_float4(__double2float_rn(uvw[3 * r]), __double2float_rn(uvw[3 * r + 1]),
                     __double2float_rn(uvw[3 * r + 2]), 0.f);
}

}  // namespace

// Which neighbouring tiles a footprint with corner (iu_local, iv_local) in
// its tile spills into: 0 none, 1 right only, 2 right and up, 3 up only.  The
// order lets the left neighbour read classes [1, 2], the lower neighbour
// [2, 3] and the diagonal one [2, 2] as contiguous key ranges.
__host__ __device__ inline int spill_class(int iu_local, int iv_local, int tile, int support) {
  const bool right = iu_local > tile - support;
  const bool up = iv_local > tile - support;
  return right ? (up ? 2 : 1) : (up ? 3 : 0);
}

namespace {

struct Footprint {
  int iu, iv, ip;
  float fu, fv, fw;
  uint32_t key;
};

__device__ __forceinline__ Footprint footprint(const DevPlan &p,
                                               const double *uvw_row,
                                               const ChannelScale &cs) {
  Footprint f;
  const double half = 0.5 * (double)p.support;
  const double U = __dmul_rn(uvw_row[0], cs.su);
  const double V = __dmul_rn(uvw_row[1], cs.sv);
  const double iu0 = ceil(__dsub_rn(U, half));
  const double iv0 = ceil(__dsub_rn(V, half));
  f.fu = __double2float_rn(__dsub_rn(iu0, U));
  f.fv = __double2float_rn(__dsub_rn(iv0, V));
  long long iu = (long long)iu0 % p.nu;
  if (iu < 0) iu += p.nu;
  long long iv = (long long)iv0 % p.nv;
  if (iv < 0) iv += p.nv;
  f.iu = (int)iu;
  f.iv = (int)iv;
  if (p.n_planes > 1) {
    const double wl = __dmul_rn(uvw_row[2], cs.sw);
    const double Pw = __dmul_rn(__dsub_rn(wl, p.w0), p.inv_dw);
    double ip0 = ceil(__dsub_rn(Pw, half));
    const double ip_max = (double)(p.n_planes - p.support);
    if (ip0 < 0.0) ip0 = 0.0;
    if (ip0 > ip_max) ip0 = ip_max;
    f.ip = (int)ip0;
    f.fw = __double2float_rn(__dsub_rn(ip0, Pw));
  } else {
    f.ip = 0;
    f.fw = 0.0f;
  }
  const uint32_t tile = (uint32_t)((f.iv / p.tile) * p.ntu + f.iu / p.tile);
  f.key = (tile * 4u + (uint32_t)spill_class(f.iu % p.tile, f.iv % p.tile, p.tile, p.support)) *
              (uint32_t)p.n_planes +
          (uint32_t)f.ip;
  return f;
}

// ---- FP32 decision of the integer footprint --------------------------------
// The corners are ceilings of FP64 values: x = (a * s) - h for u and v, and
// y = ((w * sw - w0) * inv_dw) - h for w.  The same chains in FP32 (inputs
// rounded to float, each operation rounded) differ from the FP64 values by at
// most 2^-24 times a few times the magnitudes involved (bounds below, with a
// factor 4 where 3.0001 suffices); where the FP32 value lies farther than that
// from every integer, its ceiling is the FP64 ceiling.  Otherwise the sample is
// left to the FP64 pass.
constexpr float kTwoM22 = 2.384185791015625e-07f;  // 2^-22

// ceil of x = fl64(fl64(a * s) - h) from a and s rounded to float, or false
// when the FP32 value is too close to an integer (or out of int range) to
// decide.
__device__ __forceinline__ bool ceil_decided(float a, float s, float h, int *c) {
  const float x = __fsub_rn(__fmul_rn(a, s), h);
  const float eb = kTwoM22 * (fabsf(x) + h) + 1e-6f;
  if (!(fabsf(x) < 1.0e9f)) return false;
  const float fx = floorf(x);
  const float lo = x - fx;  // exact
  if (!(lo > eb && lo < 1.0f - eb)) return false;
  *c = (int)fx + 1;
  return true;
}

// Wraps a corner into [0, n) as the FP64 path does ((c mod n) + n mod n),
// for corners within one period of the grid.
__device__ __forceinline__ bool wrap_decided(int c, int n, int *out) {
  if (c < -n || c >= 2 * n) return false;
  *out = c < 0 ? c + n : (c >= n ? c - n : c);
  return true;
}

// The footprint corner of a sample decided in FP32: the unwrapped corners
// iu0, iv0, the wrapped iu, iv and the first plane ip; false when any of them
// needs the FP64 footprint.
__device__ __forceinline__ bool corners_decided(const DevPlan &p, const float4 rf,
                                                const ChannelScale &cs, int *iu0_out,
                                                int *iv0_out, int *iu_out, int *iv_out,
                                                int *ip_out) {
  const float half = 0.5f * (float)p.support;
  int iu0, iv0, iu, iv, ip = 0;
  if (!ceil_decided(rf.x, cs.fsu, half, &iu0) || !ceil_decided(rf.y, cs.fsv, half, &iv0))
    return false;
  if (!wrap_decided(iu0, p.nu, &iu) || !wrap_decided(iv0, p.nv, &iv)) return false;
  if (p.n_planes > 1) {
    const float wl = __fmul_rn(rf.z, cs.fsw);
    const float w0 = p.w0f, idw = p.inv_dwf;
    const float d = __fsub_rn(wl, w0);
    const float pw = __fmul_rn(d, idw);
    const float y = __fsub_rn(pw, half);
    const float eb =
        kTwoM22 * (fabsf(idw) * (fabsf(wl) + fabsf(w0) + fabsf(d)) + fabsf(pw) + fabsf(y)) + 1e-6f;
    const int ip_max = p.n_planes - p.support;
    if (!(fabsf(y) < 1.0e9f)) return false;
    if (y + eb <= 0.0f) {
      ip = 0;  // ceil(y) <= 0
    } else if (y - eb > (float)(ip_max - 1)) {
      ip = ip_max;  // ceil(y) >= ip_max
    } else {
      const float fy = floorf(y);
      const float lo = y - fy;
      if (!(lo > eb && lo < 1.0f - eb)) return false;
      ip = min(max((int)fy + 1, 0), ip_max);
    }
  }
  *iu0_out = iu0;
  *iv0_out = iv0;
  *iu_out = iu;
  *iv_out = iv;
  *ip_out = ip;
  return true;
}

// Key (and corner row / first plane) of a sample decided in FP32; false
// when any of the three corners needs the FP64 footprint.
__device__ __forceinline__ bool key_decided(const DevPlan &p, const float4 rf,
                                            const ChannelScale &cs, uint32_t *key, int *iu_out,
                                            int *iv_out, int *ip_out) {
  int iu0, iv0, iu, iv, ip;
  if (!corners_decided(p, rf, cs, &iu0, &iv0, &iu, &iv, &ip)) return false;
  const int tu = p.tile == 16 ? iu >> 4 : iu / p.tile;
  const int tv = p.tile == 16 ? iv >> 4 : iv / p.tile;
  const uint32_t tile = (uint32_t)(tv * p.ntu + tu);
  *key = (tile * 4u + (uint32_t)spill_class(iu - tu * p.tile, iv - tv * p.tile, p.tile,
                                            p.support)) *
             (uint32_t)p.n_planes +
         (uint32_t)ip;
  *iu_out = iu;
  *iv_out = iv;
  *ip_out = ip;
  return true;
}

// The footprint corner inside its 16 x 16 tile as one byte: (iv mod 16) * 16
// + (iu mod 16), the minor sort key within a (tile, class, first plane) key.
__host__ __device__ __forceinline__ uint8_t corner_byte(int iu, int iv) {
  return (uint8_t)(((iv & 15) << 4) | (iu & 15));
}

__device__ __forceinline__ bool is_zero(const float2 v) {
  return v.x == 0.0f && v.y == 0.0f;
}

// Which samples take part: inversion skips zero visibilities
// (gridder_simple.h:111); a prediction mask skips samples whose byte is 0.
struct Selector {
  const float2 *vis;     // non-null: skip samples equal to 0
  const uint8_t *mask;   // non-null: skip samples with mask 0
  __device__ __forceinline__ bool operator()(int64_t e) const {
    if (vis && is_zero(vis[e])) return false;
    if (mask && mask[e] == 0) return false;
    return true;
  }
};

// Order-preserving map double -> uint64 for atomic min/max.
__device__ __forceinline__ unsigned long long dkey(double d) {
  unsigned long long b = (unsigned long long)__double_as_longlong(d);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double dkey_inv(unsigned long long k) {
  unsigned long long b = (k & 0x8000000000000000ull) ? (k & ~0x8000000000000000ull) : ~k;
  double d;
  memcpy(&d, &b, sizeof(d));
  return d;
}

struct MinOp {
  __device__ double operator()(double a, double b) const { return fmin(a, b); }
};
struct MaxOp {
  __device__ double operator()(double a, double b) const { return fmax(a, b); }
};

// With TABLE the block first divides each channel's frequency by c into
// shared memory (n_chan doubles), instead of dividing once per sample; the
// quotients are the same correctly rounded values either way.
template <bool TABLE>
__global__ void __launch_bounds__(kThreads)
    w_extent_kernel(const double *uvw, const double *freq, Selector sel,
                    int64_t n_rows, int64_t n_chan,
                    unsigned long long *out /*[3]: min key, max key, count*/) {
  extern __shared__ double fl_tab[];
  if (TABLE) {
    for (int64_t c = threadIdx.x; c < n_chan; c += blockDim.x)
      fl_tab[c] = __ddiv_rn(freq[c], kSpeedOfLight);
    __syncthreads();
  }
  double wmin = 1e300, wmax = -1e300;
  unsigned long long cnt = 0;
  const int64_t n = n_rows * n_chan;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (!sel(e)) continue;
    const int64_t r = e / n_chan, c = e - r * n_chan;
    const double fl = TABLE ? fl_tab[c] : __ddiv_rn(freq[c], kSpeedOfLight);
    const double wl = __dmul_rn(uvw[3 * r + 2], fl);
    wmin = fmin(wmin, wl);
    wmax = fmax(wmax, wl);
    ++cnt;
  }
  typedef cub::BlockReduce<double, kThreads> BR;
  typedef cub::BlockReduce<unsigned long long, kThreads> BRU;
  __shared__ union {
    typename BR::TempStorage d;
    typename BRU::TempStorage u;
  } tmp;
  const double bmin = BR(tmp.d).Reduce(wmin, MinOp());
  __syncthreads();
  const double bmax = BR(tmp.d).Reduce(wmax, MaxOp());
  __syncthreads();
  const unsigned long long bcnt = BRU(tmp.u).Sum(cnt);
  if (threadIdx.x == 0) {
    if (bcnt > 0) {
      atomicMin(&out[0], dkey(bmin));
      atomicMax(&out[1], dkey(bmax));
      atomicAdd(&out[2], bcnt);
    }
  }
}

// Rank of each channel among the channels by frequency (ties by index), and
// 1/wavelength of the channels in rank order.  1/wavelength = f / c rounded
// is non-decreasing in f, so rank order is 1/wavelength order.
__global__ void channel_rank_kernel(const double *__restrict__ freq, int n_chan, int *rank,
                                    double *by_rank) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_chan) return;
  const double f = freq[c];
  int r = 0;
  for (int j = 0; j < n_chan; ++j) {
    const double g = freq[j];
    r += (g < f || (g == f && j < c)) ? 1 : 0;
  }
  rank[c] = r;
  by_rank[r] = __ddiv_rn(f, kSpeedOfLight);
}

// The same extent as w_extent_kernel with one warp per row: the row's
// selected channels give their lowest and highest rank, and only those two
// products are formed.  fl(w x) is monotone in x (non-decreasing for w >= 0,
// non-increasing below), so they are the row's extreme products, bit for bit.
// Shared memory: n_chan doubles (1/wavelength by rank), then n_chan ints (ranks).
__global__ void __launch_bounds__(kThreads, 4)
    w_extent_rows_kernel(const double *uvw, const int *__restrict__ rank_g,
                         const double *__restrict__ by_rank_g, Selector sel, int64_t n_rows,
                         int n_chan, unsigned long long *out /*[3]: min key, max key, count*/) {
  extern __shared__ double by_rank[];
  int *rank = reinterpret_cast<int *>(by_rank + n_chan);
  for (int c = threadIdx.x; c < n_chan; c += blockDim.x) {
    by_rank[c] = by_rank_g[c];
    rank[c] = rank_g[c];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double wmin = 1e300, wmax = -1e300;
  unsigned long long cnt = 0;
  // kRows consecutive rows per warp step, their loads issued together
  constexpr int kRows = 4;
  for (int64_t r0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kRows; r0 < n_rows;
       r0 += n_warps * kRows) {
    double w[kRows];
    unsigned lo[kRows], hi[kRows], k[kRows];
#pragma unroll
    for (int j = 0; j < kRows; ++j) {
      w[j] = r0 + j < n_rows ? uvw[3 * (r0 + j) + 2] : 0.0;
      lo[j] = 0xffffffffu;
      hi[j] = 0u;
      k[j] = 0u;
    }
    // 64 channels of the kRows rows per round: every selection load of the
    // round is issued before any is used
    for (int c0 = 0; c0 < n_chan; c0 += 64) {
      bool on[kRows][2];
#pragma unroll
      for (int j = 0; j < kRows; ++j)
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int c = c0 + 32 * u + lane;
          on[j][u] = r0 + j < n_rows && c < n_chan && sel((r0 + j) * n_chan + c);
        }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int c = c0 + 32 * u + lane;
        const unsigned q = c < n_chan ? (unsigned)rank[c] : 0u;
#pragma unroll
        for (int j = 0; j < kRows; ++j) {
          if (on[j][u]) {
            lo[j] = min(lo[j], q);
            hi[j] = max(hi[j], q);
            ++k[j];
          }
        }
      }
    }
    // lane j takes row j's two products, so that the FP64 work of the kRows
    // rows is one set of warp instructions
    unsigned my_l = 0, my_h = 0, my_k = 0;
    double my_w = 0.0;
#pragma unroll
    for (int j = 0; j < kRows; ++j) {
      const unsigned l = __reduce_min_sync(0xffffffffu, lo[j]);
      const unsigned h = __reduce_max_sync(0xffffffffu, hi[j]);
      const unsigned kk = __reduce_add_sync(0xffffffffu, k[j]);
      if (lane == j) {
        my_l = l;
        my_h = h;
        my_k = kk;
        my_w = w[j];
      }
    }
    if (my_k > 0) {
      const double a = __dmul_rn(my_w, by_rank[my_l]), b = __dmul_rn(my_w, by_rank[my_h]);
      wmin = fmin(wmin, fmin(a, b));
      wmax = fmax(wmax, fmax(a, b));
      cnt += my_k;
    }
  }
  typedef cub::BlockReduce<double, kThreads> BR;
  typedef cub::BlockReduce<unsigned long long, kThreads> BRU;
  __shared__ union {
    typename BR::TempStorage d;
    typename BRU::TempStorage u;
  } tmp;
  const double bmin = BR(tmp.d).Reduce(wmin, MinOp());
  __syncthreads();
  const double bmax = BR(tmp.d).Reduce(wmax, MaxOp());
  __syncthreads();
  const unsigned long long bcnt = BRU(tmp.u).Sum(cnt);
  if (threadIdx.x == 0) {
    if (bcnt > 0) {
      atomicMin(&out[0], dkey(bmin));
      atomicMax(&out[1], dkey(bmax));
      atomicAdd(&out[2], bcnt);
    }
  }
}

__global__ void __launch_bounds__(kThreads)
    key_kernel(DevPlan p, const double *uvw, const ChannelScale *cs,
               Selector sel, int64_t n_rows, int64_t n_chan,
               uint32_t sentinel, uint32_t *keys,
               uint32_t *vals, uint32_t *counts, uint8_t *corners,
               uint32_t *pending, uint32_t *n_pending, const float4 *__restrict__ uvwf,
               uint8_t *__restrict__ minor) {
  const int64_t n = n_rows * n_chan;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  // n < 2^32 (the callers check it): 32-bit division, which needs no FP64
  const uint32_t r32 = (uint32_t)e / (uint32_t)n_chan;
  const int64_t r = r32, c = (int64_t)((uint32_t)e - r32 * (uint32_t)n_chan);
  uint32_t key = sentinel;
  uint8_t cb = 0;
  bool defer = false;
  // the row and channel terms are loaded with the selection, not after it
  const float4 rf = row_float(uvwf, uvw, r);
  const ChannelScale sc = cs[c];
  if (sel(e)) {
    int iu, iv, ip;
    if (key_decided(p, rf, sc, &key, &iu, &iv, &ip)) {
      if (corners) corners[(size_t)ip * p.nv + iv] = 1;
      cb = corner_byte(iu, iv);
    } else {
      defer = true;
    }
  }
  minor[e] = cb;
  {
    // samples the FP32 test cannot decide go to the FP64 pass (key_fix_kernel)
    const unsigned dm = __ballot_sync(__activemask(), defer);
    if (dm) {
      const int lane = threadIdx.x & 31;
      const int leader = __ffs(dm) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(n_pending, (uint32_t)__popc(dm));
      base = __shfl_sync(__activemask(), base, leader);
      if (defer) pending[base + __popc(dm & ((1u << lane) - 1u))] = (uint32_t)e;
    }
  }
  keys[e] = key;
  vals[e] = (uint32_t)e;
  if (counts && key != sentinel) {
    // warp-aggregated histogram update
    const unsigned active = __activemask();
    const unsigned peers = __match_any_sync(active, key);
    const int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(&counts[key], __popc(peers));
  }
}

// FP64 footprints of the samples key_kernel deferred: key, corner mark and
// (counts non-null) histogram count.
__global__ void __launch_bounds__(kThreads)
    key_fix_kernel(DevPlan p, const double *uvw, const ChannelScale *cs, int64_t n_chan,
                   const uint32_t *__restrict__ pending, const uint32_t *__restrict__ n_pending,
                   uint32_t *keys, uint32_t *counts, uint8_t *corners, uint8_t *minor) {
  const uint32_t n = *n_pending;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t e = pending[i];
    const uint32_t r32 = e / (uint32_t)n_chan;
    const int64_t r = r32, c = (int64_t)(e - r32 * (uint32_t)n_chan);
    const Footprint f = footprint(p, uvw + 3 * r, cs[c]);
    keys[e] = f.key;
    minor[e] = corner_byte(f.iu, f.iv);
    if (corners) corners[(size_t)f.ip * p.nv + f.iv] = 1;
    if (counts) atomicAdd(&counts[f.key], 1u);
  }
}

// ---------------- stable LSD radix sort, 8-bit digits ----------------------
constexpr int kSortItems = 16;
constexpr int kSortTile = kThreads * kSortItems;  // 4096 elements per block

// digits: when non-null, element i's digit is digits[i] instead of the key's
// 8 bits at `shift` (the corner pass).
__global__ void __launch_bounds__(kThreads)
    radix_hist_kernel(const uint32_t *keys, const uint8_t *__restrict__ digits, int64_t n,
                      int shift, uint32_t *hist, int64_t n_blocks, bool drop, uint32_t drop_key) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortTile;
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const int64_t i = base + r * kThreads + threadIdx.x;
    if (i < n) {
      const uint32_t k = keys[i];
      const uint32_t d = digits ? (uint32_t)digits[i] : (k >> shift) & 255u;
      if (!(drop && k == drop_key)) atomicAdd(&h[d], 1u);
    }
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * n_blocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one 8-bit digit.  Each block first orders its tile of
// kSortTile elements by digit in shared memory (stable: rank by round, warp
// and lane), then writes each digit's run to its global range, so that
// consecutive threads write consecutive addresses.  hist holds the exclusive
// scan of the per-(digit, block) counts (digit-major); a tile's own count of
// digit d is the difference to the next entry (n_kept after the last).  With
// drop, elements whose key is drop_key take no part (the histogram skipped
// them too) and n_kept elements come out.
__global__ void __launch_bounds__(kThreads)
    radix_scatter_kernel(const uint32_t *keys_in, const uint32_t *vals_in,
                         const uint8_t *__restrict__ digits, int64_t n, int shift,
                         const uint32_t *hist, int64_t n_blocks, uint32_t *keys_out,
                         uint32_t *vals_out, bool drop, uint32_t drop_key, uint32_t n_kept) {
  __shared__ uint32_t base[256];    // global position of the tile's first element of digit d
  __shared__ uint32_t tstart[256];  // first position of digit d in the tile's sorted order
  __shared__ uint32_t run[256];     // elements of digit d placed by earlier rounds
  __shared__ uint32_t wcnt[kThreads / 32][256];
  __shared__ uint32_t wsum[kThreads / 32];
  __shared__ uint32_t tile_kept;
  __shared__ uint32_t skey[kSortTile], sval[kSortTile];
  __shared__ uint8_t sdig[kSortTile];
  static_assert(kThreads == 256, "one thread per digit");
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tile0 = (int64_t)blockIdx.x * kSortTile;
  const int tile_n = (int)min((int64_t)kSortTile, n - tile0);
  {
    const int64_t at = (int64_t)threadIdx.x * n_blocks + blockIdx.x;
    const uint32_t b0 = hist[at];
    const uint32_t b1 = (threadIdx.x == 255 && blockIdx.x == n_blocks - 1) ? n_kept
                                                                           : hist[at + 1];
    base[threadIdx.x] = b0;
    run[threadIdx.x] = 0;
    // exclusive scan of the tile's digit counts (one digit per thread)
    const uint32_t cnt = b1 - b0;
    uint32_t x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    tstart[threadIdx.x] = before + x - cnt;
    if (threadIdx.x == 255) tile_kept = before + x;
  }
  const unsigned lt_mask = (1u << lane) - 1u;
  for (int r = 0; r < kSortItems; ++r) {
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const int t = r * kThreads + threadIdx.x;
    bool valid = t < tile_n;
    uint32_t key = 0, val = 0, d = 256;
    if (valid) {
      key = keys_in[tile0 + t];
      val = vals_in[tile0 + t];
      d = digits ? (uint32_t)digits[tile0 + t] : (key >> shift) & 255u;
      if (drop && key == drop_key) {
        valid = false;
        d = 256;
      }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & lt_mask);
    if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    {
      uint32_t acc = run[threadIdx.x];
#pragma unroll
      for (int w = 0; w < kThreads / 32; ++w) {
        const uint32_t c = wcnt[w][threadIdx.x];
        wcnt[w][threadIdx.x] = acc;
        acc += c;
      }
      run[threadIdx.x] = acc;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = tstart[d] + wcnt[warp][d] + rank;
      skey[pos] = key;
      sval[pos] = val;
      sdig[pos] = (uint8_t)d;
    }
    __syncthreads();  // wcnt is cleared for the next round
  }
  for (int j = threadIdx.x; j < (int)tile_kept; j += kThreads) {
    const uint32_t d = sdig[j];
    const uint32_t out = base[d] + ((uint32_t)j - tstart[d]);
    keys_out[out] = skey[j];
    vals_out[out] = sval[j];
  }
}

// ---------------- stable LSD radix sort, one kernel per 8-bit digit ----------
// The same sort as above without the per-pass histogram and scan.  The digit
// totals of every pass are counted beforehand (the corner byte by
// corner_count_kernel, the key bytes during the first pass).  Blocks take
// tiles of kThreads * ITEMS elements in order from a counter, so every lower
// tile belongs to a block that has already started.  A block ranks its tile's
// elements by digit (each warp a contiguous run of 32 * ITEMS elements, with
// warp-private counts), publishes the tile's count of each digit, and adds up
// the counts of the lower tiles by looking back over their published words:
// a tile first publishes its own count (an aggregate), then, once its
// look-back has ended, the inclusive sum over all tiles up to itself (a
// prefix); a look-back stops at the first prefix it meets and reads
// kSweepWindow lower tiles per round trip.  This is the single-pass prefix
// scan with decoupled look-back (Merrill and Garland, 2016) applied per digit,
// as in the Onesweep sort (Adinets and Merrill, 2022).  Each published word
// carries its flag and count together, so relaxed loads and stores suffice.
// A wait on a lower tile gives up after kSweepSpinLimit polls and reports
// through the caller's flag word.
constexpr uint64_t kSweepAggregate = 1ull << 62;
constexpr uint64_t kSweepPrefix = 2ull << 62;
constexpr uint64_t kSweepFlags = 3ull << 62;
constexpr uint32_t kSweepSpinLimit = 1u << 20;
constexpr int kSweepWindow = 8;        // lower tiles read per look-back step
constexpr int kSweepMaxKeyPasses = 4;  // 32-bit keys
// the library's configuration: elements per thread, resident blocks per SM
constexpr int kSweepItems = 12;
constexpr int kSweepMinBlocks = 3;

template <int ITEMS>
__host__ __device__ constexpr int sweep_tile() {
  return kThreads * ITEMS;
}
// dynamic shared memory: warp counts, next-pass counts, tile keys and values, tile digits
template <int ITEMS>
__host__ __device__ constexpr size_t sweep_smem() {
  return sizeof(uint32_t) *
             ((kThreads / 32) * 256 + kSweepMaxKeyPasses * 256 + 2 * sweep_tile<ITEMS>()) +
         sweep_tile<ITEMS>();
}

__device__ __forceinline__ void store_relaxed_u64(uint64_t *p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t load_relaxed_u64(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Exclusive scan of one value per thread over the block (kThreads threads);
// *total receives the sum.  Ends with a barrier.
__device__ __forceinline__ uint32_t sweep_block_scan(uint32_t v, uint32_t *wsum,
                                                     uint32_t *total) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  uint32_t before = 0, all = 0;
#pragma unroll
  for (int w = 0; w < kThreads / 32; ++w) {
    const uint32_t s = wsum[w];
    if (w < warp) before += s;
    all += s;
  }
  *total = all;
  __syncthreads();
  return before + x - v;
}

// Counts of the corner byte over the elements whose key is not drop_key, and
// their number in *kept.
__global__ void __launch_bounds__(kThreads)
    corner_count_kernel(const uint32_t *__restrict__ keys, const uint8_t *__restrict__ minor,
                        int64_t n, uint32_t drop_key, uint32_t *totals, uint32_t *kept) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t n4 = n / 4, stride = (int64_t)gridDim.x * kThreads;
  const uint4 *k4 = reinterpret_cast<const uint4 *>(keys);
  const uint32_t *m4 = reinterpret_cast<const uint32_t *>(minor);
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n4; i += stride) {
    const uint4 k = __ldg(k4 + i);
    const uint32_t m = __ldg(m4 + i);  // bytes 4i .. 4i+3, the first in the low bits
    if (k.x != drop_key) atomicAdd(&h[m & 255u], 1u);
    if (k.y != drop_key) atomicAdd(&h[(m >> 8) & 255u], 1u);
    if (k.z != drop_key) atomicAdd(&h[(m >> 16) & 255u], 1u);
    if (k.w != drop_key) atomicAdd(&h[m >> 24], 1u);
  }
  for (int64_t i = 4 * n4 + (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += stride)
    if (keys[i] != drop_key) atomicAdd(&h[minor[i]], 1u);
  __syncthreads();
  const uint32_t c = h[threadIdx.x];
  if (c) atomicAdd(&totals[threadIdx.x], c);
  uint32_t sum = c;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(kept, sum);
}

// Number of elements of each key, from the keys in sorted order (equal keys
// are consecutive: one warp-aggregated atomic per key and warp, on counters
// in increasing order).
__global__ void __launch_bounds__(kThreads)
    count_sorted_keys_kernel(const uint32_t *__restrict__ keys, int64_t n, uint32_t *counts) {
  const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = keys[i];
  const unsigned peers = __match_any_sync(__activemask(), k);
  if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&counts[k], (uint32_t)__popc(peers));
}

// Status words of kSweepWindow lower tiles q, q - 1, ... for digit t (below
// tile 0: a prefix of zero).
__device__ __forceinline__ void sweep_window(const uint64_t *status, int64_t q, int t,
                                             uint64_t (&x)[kSweepWindow]) {
#pragma unroll
  for (int j = 0; j < kSweepWindow; ++j)
    x[j] = q - j >= 0 ? load_relaxed_u64(status + (q - j) * 256 + t) : kSweepPrefix;
}

// One stable pass over the n elements of (keys_in, vals_in) by the 8-bit digit
// at `shift` (FIRST: by minor[i], leaving out the elements whose key is
// drop_key, and counting the kept keys' n_next bytes into next_totals for the
// later passes).  totals: the pass's count of each digit.  status: 256 words
// per tile, zero at launch; tile_counter zero at launch.
template <bool FIRST, int ITEMS, int MINB>
__global__ void __launch_bounds__(kThreads, MINB)
    sweep_kernel(const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
                 const uint8_t *__restrict__ minor, int64_t n, int shift, uint32_t drop_key,
                 const uint32_t *__restrict__ totals, uint64_t *status, uint32_t *tile_counter,
                 uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out,
                 uint32_t *next_totals, int n_next, unsigned *wait_flags) {
  constexpr int kTile = sweep_tile<ITEMS>(), kRun = 32 * ITEMS;
  static_assert(kRun <= 0xffff, "warp ranks are 16-bit");
  extern __shared__ uint32_t sweep_smem[];
  uint32_t(*wcnt)[256] = reinterpret_cast<uint32_t(*)[256]>(sweep_smem);
  uint32_t(*ncnt)[256] = reinterpret_cast<uint32_t(*)[256]>(sweep_smem + (kThreads / 32) * 256);
  uint32_t *skey = sweep_smem + (kThreads / 32 + kSweepMaxKeyPasses) * 256;
  uint32_t *sval = skey + kTile;
  uint8_t *sdig = reinterpret_cast<uint8_t *>(sval + kTile);
  __shared__ uint32_t gbase[256], wsum[kThreads / 32];
  __shared__ uint32_t s_tile, s_kept;
  static_assert(kThreads == 256, "one thread per digit");
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, t = threadIdx.x;
  const unsigned lt = (1u << lane) - 1u;
  const int64_t n_tiles = (n + kTile - 1) / kTile;
  if (FIRST)
    for (int j = 0; j < kSweepMaxKeyPasses; ++j) ncnt[j][t] = 0;
  // the pass's first position of each digit
  uint32_t unused;
  const uint32_t dstart = sweep_block_scan(totals[t], wsum, &unused);
  for (;;) {
    if (t == 0) s_tile = atomicAdd(tile_counter, 1u);
    for (int i = lane; i < 256; i += 32) wcnt[warp][i] = 0;
    __syncthreads();
    const int64_t tile = s_tile;
    if (tile >= n_tiles) break;
    const int64_t run0 = tile * kTile + warp * kRun;
    uint32_t kr[ITEMS], vr[ITEMS], dr[ITEMS];
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
      const int64_t i = run0 + r * 32 + lane;
      uint32_t d = 256;  // no element
      kr[r] = 0;
      vr[r] = 0;
      if (i < n) {
        kr[r] = keys_in[i];
        vr[r] = vals_in[i];
        if (FIRST) {
          const uint32_t m = minor[i];  // loaded with the key, not after it
          d = kr[r] != drop_key ? m : 256u;
        } else {
          d = (kr[r] >> shift) & 255u;
        }
      }
      dr[r] = d;
    }
    // rank within the warp's run: earlier rounds, then lower lanes
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
      const uint32_t d = dr[r];
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      uint32_t before = 0;
      if (d < 256) before = wcnt[warp][d];
      __syncwarp();
      if (d < 256 && (peers & lt) == 0) wcnt[warp][d] = before + __popc(peers);
      __syncwarp();
      dr[r] = (d << 16) | (before + __popc(peers & lt));
    }
    __syncthreads();
    // thread t: digit t's offsets of the warps and the tile's count
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) {
      const uint32_t c = wcnt[w][t];
      wcnt[w][t] = cnt;
      cnt += c;
    }
    uint64_t *mine = status + tile * 256 + t;
    store_relaxed_u64(mine, (tile == 0 ? kSweepPrefix : kSweepAggregate) | cnt);
    // the first look-back window is in flight while the tile is placed
    int64_t q = tile - 1;
    uint64_t x[kSweepWindow];
    if (tile > 0) sweep_window(status, q, t, x);
    uint32_t kept;
    const uint32_t first = sweep_block_scan(cnt, wsum, &kept);
    // each warp's first tile position of digit t
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) wcnt[w][t] += first;
    if (t == 0) s_kept = kept;
    __syncthreads();  // tile positions of every digit
    // the tile in digit order in shared memory
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
      const uint32_t d = dr[r] >> 16;
      if (d < 256) {
        const uint32_t pos = wcnt[warp][d] + (dr[r] & 0xffffu);
        skey[pos] = kr[r];
        sval[pos] = vr[r];
        sdig[pos] = (uint8_t)d;
      }
    }
    // digit t's count over the lower tiles: tiles q, q - 1, ... are added
    // while they have published, up to the first prefix; an unpublished tile
    // is read again in the next window
    uint32_t excl = 0;
    if (tile > 0) {
      uint32_t polls = 0;
      for (;;) {
        int added = 0;
        bool done = false, stop = false;
#pragma unroll
        for (int j = 0; j < kSweepWindow; ++j) {
          const uint64_t f = x[j] & kSweepFlags;
          if (!stop) {
            if (f == 0) {
              stop = true;
            } else {
              excl += (uint32_t)x[j];
              ++added;
              if (f == kSweepPrefix) done = stop = true;
            }
          }
        }
        if (done) break;
        q -= added;
        if (added == 0) {
          if (++polls > kSweepSpinLimit) {
            atomicOr(wait_flags, 1u);
            break;
          }
          if (polls > 32) __nanosleep(64);
        }
        sweep_window(status, q, t, x);
      }
      store_relaxed_u64(mine, kSweepPrefix | (uint32_t)(excl + cnt));
    }
    // output position of tile position j of digit d: gbase[d] + j (the
    // tile's first position of the digit taken off, modulo 2^32)
    gbase[t] = dstart + excl - first;
    __syncthreads();
    const uint32_t tile_kept = s_kept;
    for (uint32_t j = t; j < tile_kept; j += kThreads) {
      const uint32_t d = sdig[j];
      const uint32_t o = gbase[d] + j;
      const uint32_t k = skey[j];
      keys_out[o] = k;
      vals_out[o] = sval[j];
      // the key bytes of the later passes, counted in corner order (in input
      // order equal bytes bunch up in a warp and their atomics collide)
      if (FIRST)
        for (int b = 0; b < n_next; ++b) atomicAdd(&ncnt[b][(k >> (8 * b)) & 255u], 1u);
    }
    __syncthreads();  // the next tile reuses the shared buffers
  }
  if (FIRST)
    for (int b = 0; b < n_next; ++b)
      if (ncnt[b][t]) atomicAdd(&next_totals[b * 256 + t], ncnt[b][t]);
}

// Footprint of a record: corners decided in FP32 where possible (see
// key_decided), fractions from the FP64 coordinates; identical to footprint().
__device__ __forceinline__ Footprint record_footprint(const DevPlan &p, const double *row,
                                                      const float4 rf, const ChannelScale &cs,
                                                      double *wl_out) {
  const float half = 0.5f * (float)p.support;
  int iu0, iv0, iu, iv;
  bool ok = ceil_decided(rf.x, cs.fsu, half, &iu0) && ceil_decided(rf.y, cs.fsv, half, &iv0) &&
            wrap_decided(iu0, p.nu, &iu) && wrap_decided(iv0, p.nv, &iv);
  Footprint f;
  double wl = 0.0, pw = 0.0;
  int ip = 0;
  if (ok && p.n_planes > 1) {
    wl = __dmul_rn(row[2], cs.sw);
    pw = __dmul_rn(__dsub_rn(wl, p.w0), p.inv_dw);
    const float wlf = __fmul_rn(rf.z, cs.fsw);
    const float w0 = p.w0f, idw = p.inv_dwf;
    const float d = __fsub_rn(wlf, w0);
    const float pwf = __fmul_rn(d, idw);
    const float y = __fsub_rn(pwf, half);
    const float eb =
        kTwoM22 * (fabsf(idw) * (fabsf(wlf) + fabsf(w0) + fabsf(d)) + fabsf(pwf) + fabsf(y)) +
        1e-6f;
    const int ip_max = p.n_planes - p.support;
    if (!(fabsf(y) < 1.0e9f)) {
      ok = false;
    } else if (y + eb <= 0.0f) {
      ip = 0;
    } else if (y - eb > (float)(ip_max - 1)) {
      ip = ip_max;
    } else {
      const float fy = floorf(y);
      const float lo = y - fy;
      if (lo > eb && lo < 1.0f - eb)
        ip = min(max((int)fy + 1, 0), ip_max);
      else
        ok = false;
    }
  }
  if (!ok) {
    *wl_out = __dmul_rn(row[2], cs.sw);
    return footprint(p, row, cs);
  }
  f.iu = iu;
  f.iv = iv;
  f.fu = __double2float_rn(__dsub_rn((double)iu0, __dmul_rn(row[0], cs.su)));
  f.fv = __double2float_rn(__dsub_rn((double)iv0, __dmul_rn(row[1], cs.sv)));
  if (p.n_planes > 1) {
    f.ip = ip;
    f.fw = __double2float_rn(__dsub_rn((double)ip, pw));
  } else {
    f.ip = 0;
    f.fw = 0.0f;
    wl = __dmul_rn(row[2], cs.sw);
  }
  f.key = 0;  // not needed for records
  *wl_out = wl;
  return f;
}

// Writes record s as float4 pairs: (re, im, fu, fv), (fw, iu, iv, ip).
__device__ __forceinline__ void store_record(VisRecord *rec, int64_t s, const float2 *vis,
                                             uint32_t e, float sn, float cn, float fu, float fv,
                                             float fw, int iu, int iv, int ip) {
  float re, im;
  if (vis) {
    const float2 v = vis[e];
    re = v.x * cn + v.y * sn;
    im = v.y * cn - v.x * sn;
  } else {
    re = cn;
    im = -sn;
  }
  reinterpret_cast<float4 *>(rec + s)[0] = make_float4(re, im, fu, fv);
  reinterpret_cast<float4 *>(rec + s)[1] =
      make_float4(fw, __int_as_float(iu), __int_as_float(iv), __int_as_float(ip));
}

// Record s (sample e) with the fractions and the phase argument from the FP64
// chains.  SHIFT: the image has an l or m shift (else the phase needs only w).
template <bool SHIFT>
__device__ __forceinline__ void record_fp64(const DevPlan &p, const double *uvw,
                                            const ChannelScale *cs, const float2 *vis,
                                            int64_t n_chan, uint32_t e, int64_t s,
                                            VisRecord *rec, const float4 *uvwf) {
  const uint32_t r = e / (uint32_t)n_chan, c = e - r * (uint32_t)n_chan;  // e < 2^32
  const double *row = uvw + 3 * (size_t)r;
  const ChannelScale sc = cs[c];
  double wl;
  const Footprint f = record_footprint(p, row, row_float(uvwf, uvw, r), sc, &wl);
  // shift phase theta = u l_shift + v m_shift + w c_n (turns), FP64 argument,
  // reduced to [-1/2, 1/2] before the FP32 sincos.  Without shifts the first
  // two terms are zero and theta = fl(w f / c) c_n, the same value.
  // (every step rounded as written: the float-float pass reproduces this chain)
  double t = __dmul_rn(wl, p.nm1_center);
  if (SHIFT) {
    const double fl = sc.sw;
    const double tuv = __dadd_rn(__dmul_rn(__dmul_rn(row[0], fl), p.l_shift),
                                 __dmul_rn(__dmul_rn(row[1], fl), p.m_shift));
    t = __dadd_rn(tuv, t);
  }
  t -= rint(t);
  float sn, cn;
  sincospif(2.0f * (float)t, &sn, &cn);
  store_record(rec, s, vis, e, sn, cn, f.fu, f.fv, f.fw, f.iu, f.iv, f.ip);
}

template <bool SHIFT>
__global__ void __launch_bounds__(kThreads)
    record_kernel(DevPlan p, const double *uvw, const ChannelScale *cs,
                  const float2 *vis, int64_t n_chan, const uint32_t *perm,
                  int64_t n_out, VisRecord *rec, const float4 *__restrict__ uvwf) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_out) return;
  record_fp64<SHIFT>(p, uvw, cs, vis, n_chan, perm[s], s, rec, uvwf);
}

// Records from float-float arithmetic (record_ff.cuh):
// the corners decided in FP32 as key_kernel decides them, the fractions and
// the phase argument where the error bound proves them equal to the FP64
// chains.  Each block takes kRecordBlock consecutive records and lists the
// ones it cannot decide in its own slice of `pending` (block b's entries from
// b * kRecordBlock, their number in counts[b]); record_fix_kernel does those
// in FP64.
constexpr int kRecordBlock = 4 * kThreads;

template <bool SHIFT>
__global__ void __launch_bounds__(kThreads)
    record_ff_kernel(DevPlan p, const ChannelScale *__restrict__ cs, const float2 *vis,
                     int64_t n_chan, const uint32_t *__restrict__ perm, int64_t n_out,
                     VisRecord *rec, const float4 *__restrict__ uvwf,
                     const float4 *__restrict__ uvwl, uint32_t *__restrict__ pending,
                     uint32_t *__restrict__ counts) {
  __shared__ uint32_t n_left;
  if (threadIdx.x == 0) n_left = 0;
  __syncthreads();
  const int64_t b0 = (int64_t)blockIdx.x * kRecordBlock;
  const ff::PlanPairs pp{ff::Pair{p.w0f, p.w0l}, ff::Pair{p.inv_dwf, p.inv_dwl},
                         ff::Pair{p.nm1_center_f, p.nm1_center_l},
                         ff::Pair{p.l_shift_f, p.l_shift_l}, ff::Pair{p.m_shift_f, p.m_shift_l},
                         p.n_planes > 1, SHIFT};
  for (int k = 0; k < kRecordBlock / kThreads; ++k) {
    const int64_t s = b0 + k * kThreads + threadIdx.x;
    if (s >= n_out) break;
    const uint32_t e = perm[s];
    const uint32_t r = e / (uint32_t)n_chan, c = e - r * (uint32_t)n_chan;
    const float4 hi = __ldg(uvwf + r), lo = __ldg(uvwl + r);
    const ChannelScale sc = cs[c];
    int iu0, iv0, iu, iv, ip;
    float fu, fv, fw, arg;
    const bool ok =
        corners_decided(p, hi, sc, &iu0, &iv0, &iu, &iv, &ip) &&
        ff::decide(ff::Pair{hi.x, lo.x}, ff::Pair{hi.y, lo.y}, ff::Pair{hi.z, lo.z},
                   ff::Scales{ff::Pair{sc.fsu, sc.lsu}, ff::Pair{sc.fsv, sc.lsv},
                              ff::Pair{sc.fsw, sc.lsw}},
                   pp, iu0, iv0, ip, &fu, &fv, &fw, &arg);
    if (!ok) {
      pending[b0 + atomicAdd(&n_left, 1u)] = (uint32_t)s;
      continue;
    }
    float sn, cn;
    sincospif(2.0f * arg, &sn, &cn);
    store_record(rec, s, vis, e, sn, cn, fu, fv, fw, iu, iv, ip);
  }
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = n_left;
}

// The records record_ff_kernel left undecided, in FP64: one warp per record
// block's slice, so that the FP64 chains run with the warp's lanes full.
template <bool SHIFT>
__global__ void __launch_bounds__(kThreads)
    record_fix_kernel(DevPlan p, const double *uvw, const ChannelScale *cs, const float2 *vis,
                      int64_t n_chan, const uint32_t *__restrict__ perm, int64_t n_blocks,
                      VisRecord *rec, const float4 *__restrict__ uvwf,
                      const uint32_t *__restrict__ pending, const uint32_t *__restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t b = w0; b < n_blocks; b += n_warps) {
    const uint32_t cnt = counts[b];
    for (uint32_t i = lane; i < cnt; i += 32) {
      const uint32_t s = pending[b * kRecordBlock + i];
      record_fp64<SHIFT>(p, uvw, cs, vis, n_chan, perm[s], s, rec, uvwf);
    }
  }
}

// ---------------- row occupancy ----------------------------------------------
constexpr int kOccThreads = 1024;

// Plane q's rows covered by a footprint: a footprint with corner (ip, iv)
// covers planes ip .. ip + W - 1 and rows iv .. iv + W - 1 (cyclically), so
// row r of plane q is covered when a corner lies on one of the planes
// q - W + 1 .. q and rows r - W + 1 .. r.  One block per plane.
__global__ void __launch_bounds__(kOccThreads)
    row_flags_kernel(const uint8_t *__restrict__ corners, int nv, int W,
                     uint8_t *__restrict__ flags, uint32_t *__restrict__ counts) {
  extern __shared__ uint8_t any_plane[];  // [nv]: corners of planes q - W + 1 .. q
  __shared__ uint32_t total;
  const int q = blockIdx.x;
  if (threadIdx.x == 0) total = 0;
  for (int r = threadIdx.x; r < nv; r += blockDim.x) {
    uint8_t a = 0;
    for (int k = 0; k < W && k <= q; ++k) a |= corners[(size_t)(q - k) * nv + r];
    any_plane[r] = a;
  }
  __syncthreads();
  uint32_t cnt = 0;
  for (int r = threadIdx.x; r < nv; r += blockDim.x) {
    uint8_t f = 0;
    for (int k = 0; k < W; ++k) {
      int rr = r - k;
      while (rr < 0) rr += nv;
      f |= any_plane[rr];
    }
    flags[(size_t)q * nv + r] = f ? 1 : 0;
    cnt += f ? 1u : 0u;
  }
  if (cnt) atomicAdd(&total, cnt);
  __syncthreads();
  if (threadIdx.x == 0) counts[q] = total;
}

// Compacts plane q's flagged rows into list[start[q] ..], in row order;
// start[q] is the sum of the earlier planes' counts.  One block per plane.
__global__ void __launch_bounds__(kOccThreads)
    row_list_kernel(const uint8_t *__restrict__ flags, const uint32_t *__restrict__ counts,
                    int n_planes, int nv, uint32_t *__restrict__ start,
                    uint32_t *__restrict__ list) {
  __shared__ uint32_t s_base;
  __shared__ uint32_t warp_tot[kOccThreads / 32];
  const int q = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  uint32_t part = 0;
  for (int k = threadIdx.x; k < q; k += blockDim.x) part += counts[k];
  if (part) atomicAdd(&s_base, part);
  __syncthreads();
  uint32_t base = s_base;
  if (threadIdx.x == 0) {
    start[q] = base;
    if (q == n_planes - 1) start[n_planes] = base + counts[q];
  }
  for (int r0 = 0; r0 < nv; r0 += blockDim.x) {
    const int r = r0 + threadIdx.x;
    const bool f = r < nv && flags[(size_t)q * nv + r] != 0;
    const unsigned m = __ballot_sync(0xffffffffu, f);
    if (lane == 0) warp_tot[warp] = __popc(m);
    __syncthreads();
    uint32_t before = 0, all = 0;
    for (int w = 0; w < n_warps; ++w) {
      const uint32_t t = warp_tot[w];
      before += w < warp ? t : 0u;
      all += t;
    }
    if (f) list[base + before + __popc(m & ((1u << lane) - 1u))] = (uint32_t)q * (uint32_t)nv + r;
    base += all;
    __syncthreads();
  }
}

// Flags, counts, starts and the row list from the corners key_kernel marked.
void build_row_occupancy(const RowOccupancy &o, int W, cudaStream_t s) {
  if (o.n_planes == 0) return;
  ensure_dynamic_smem((const void *)row_flags_kernel, (size_t)o.nv);
  row_flags_kernel<<<o.n_planes, kOccThreads, o.nv, s>>>(o.corners(), o.nv, W, o.flags(),
                                                          o.counts());
  check_launch("row_flags_kernel");
  row_list_kernel<<<o.n_planes, kOccThreads, 0, s>>>(o.flags(), o.counts(), o.n_planes, o.nv,
                                                      o.start(), o.list());
  check_launch("row_list_kernel");
}

unsigned grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

namespace {
// Stable LSD radix sort of (key, value) pairs by (key over `bits` bits, minor
// byte): the first pass orders by minor[i] (element i of the unsorted input),
// the following ones by the key's 8-bit digits.  The first pass drops the
// elements whose key is `sentinel` (samples that take no part), so the n_kept
// others come out; kin / vin end up naming the sorted buffers.  scan(d, n) is
// an exclusive scan of n uint32 values in place.  Three kernels per pass (a
// per-tile histogram, the scan, a scatter) with scratch the caller sizes: the
// allocation-free bucketing uses it; bucket_visibilities uses sweep_sort_kept,
// which gives the same order.
template <class Scan>
void radix_sort_kept(uint32_t *&kin, uint32_t *&vin, uint32_t *&kout, uint32_t *&vout,
                     const uint8_t *minor, int64_t n, uint32_t n_kept, int bits,
                     uint32_t sentinel, uint32_t *hist, Scan scan, cudaStream_t s) {
  int64_t cur = n;
  for (int pass = -1, shift = 0; shift < bits && cur > 0 && n_kept > 0; ++pass) {
    const bool drop = pass == -1;
    const uint8_t *digits = pass == -1 ? minor : nullptr;
    const int64_t n_blocks = (cur + kSortTile - 1) / kSortTile;
    radix_hist_kernel<<<(unsigned)n_blocks, kThreads, 0, s>>>(kin, digits, cur, shift, hist,
                                                              n_blocks, drop, sentinel);
    check_launch("radix_hist_kernel");
    scan(hist, 256 * n_blocks);
    radix_scatter_kernel<<<(unsigned)n_blocks, kThreads, 0, s>>>(
        kin, vin, digits, cur, shift, hist, n_blocks, kout, vout, drop, sentinel, n_kept);
    check_launch("radix_scatter_kernel");
    std::swap(kin, kout);
    std::swap(vin, vout);
    cur = n_kept;
    if (pass >= 0) shift += 8;
  }
}

// 64-bit words of look-back status that sweep_sort_kept needs for n elements
// (tiles of kThreads * ITEMS), followed by sweep_counter_words() words of counters.
template <int ITEMS = kSweepItems>
int64_t sweep_status_words(int64_t n) {
  return 256 * ((n + sweep_tile<ITEMS>() - 1) / sweep_tile<ITEMS>());
}
// counters: one tile counter per pass, the kept count, then 256 digit totals per pass
constexpr int64_t kSweepKeptWord = 6;
constexpr int64_t sweep_counter_words() { return 8 + (1 + kSweepMaxKeyPasses) * 256; }

// First step of sweep_sort_kept: zeroes the counters and counts the corner
// bytes and the number of kept elements (counters word kSweepKeptWord).
template <int ITEMS = kSweepItems>
void sweep_count(const uint32_t *keys, const uint8_t *minor, int64_t n, uint32_t sentinel,
                 uint64_t *status, cudaStream_t s) {
  uint32_t *counters = (uint32_t *)(status + sweep_status_words<ITEMS>(n));
  WGPU_CUDA(cudaMemsetAsync(counters, 0, sizeof(uint32_t) * sweep_counter_words(), s));
  if (n <= 0) return;
  corner_count_kernel<<<sm_count() * 4, kThreads, 0, s>>>(keys, minor, n, sentinel, counters + 8,
                                                          counters + kSweepKeptWord);
  check_launch("corner_count_kernel");
}
template <int ITEMS = kSweepItems>
const uint32_t *sweep_kept_word(const uint64_t *status, int64_t n) {
  return (const uint32_t *)(status + sweep_status_words<ITEMS>(n)) + kSweepKeptWord;
}

// The same sort as radix_sort_kept with one sweep_kernel per digit, after
// sweep_count on the same keys and status; n_kept is the count it made.
// status: sweep_status_words<ITEMS>(n) words, then the counters; wait_flags:
// the word an expired look-back wait is reported in.
template <int ITEMS = kSweepItems, int MINB = kSweepMinBlocks>
void sweep_sort_kept(uint32_t *&kin, uint32_t *&vin, uint32_t *&kout, uint32_t *&vout,
                     const uint8_t *minor, int64_t n, uint32_t n_kept, int bits,
                     uint32_t sentinel, uint64_t *status, unsigned *wait_flags,
                     cudaStream_t s) {
  if (n <= 0 || n_kept == 0) return;
  const int n_key_passes = (bits + 7) / 8;
  if (n_key_passes > kSweepMaxKeyPasses)
    throw Error(WGPU_ERR_INVALID, "sort key wider than 32 bits");
  constexpr int kTile = sweep_tile<ITEMS>();
  constexpr size_t kSmem = sweep_smem<ITEMS>();
  uint32_t *counters = (uint32_t *)(status + sweep_status_words<ITEMS>(n));
  uint32_t *tile_counters = counters;  // one per pass
  uint32_t *totals = counters + 8;     // per pass, 256 digits
  auto first = sweep_kernel<true, ITEMS, MINB>;
  auto later = sweep_kernel<false, ITEMS, MINB>;
  ensure_dynamic_smem((const void *)first, kSmem);
  ensure_dynamic_smem((const void *)later, kSmem);
  int64_t cur = n;
  for (int pass = 0; pass <= n_key_passes; ++pass) {
    const int64_t tiles = (cur + kTile - 1) / kTile;
    WGPU_CUDA(cudaMemsetAsync(status, 0, sizeof(uint64_t) * 256 * tiles, s));
    int per_sm = 0;
    WGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, pass == 0 ? (const void *)first : (const void *)later, kThreads, kSmem));
    const unsigned blocks =
        (unsigned)std::min<int64_t>(tiles, (int64_t)sm_count() * std::max(per_sm, 1));
    if (pass == 0) {
      first<<<blocks, kThreads, kSmem, s>>>(kin, vin, minor, cur, 0, sentinel, totals, status,
                                            tile_counters, kout, vout, totals + 256,
                                            n_key_passes, wait_flags);
    } else {
      later<<<blocks, kThreads, kSmem, s>>>(kin, vin, nullptr, cur, 8 * (pass - 1), sentinel,
                                            totals + 256 * pass, status, tile_counters + pass,
                                            kout, vout, nullptr, 0, wait_flags);
    }
    check_launch("sweep_kernel");
    std::swap(kin, kout);
    std::swap(vin, vout);
    cur = n_kept;
  }
}
}  // namespace

RowOccupancy copy_row_occupancy(const RowOccupancy &rows, void *dst, cudaStream_t s) {
  RowOccupancy o = rows;
  if (!rows.buf) return o;
  o.buf = (uint8_t *)dst;
  WGPU_CUDA(cudaMemcpyAsync(o.buf, rows.buf, rows.bytes(), cudaMemcpyDeviceToDevice, s));
  return o;
}

size_t w_extent_scratch_bytes(int64_t n_chan) {
  return 64 + (sizeof(int) + sizeof(double)) * (size_t)(n_chan + 2);
}

void compute_w_extent(const double *d_uvw, const double *d_freq,
                      const float *d_vis, const uint8_t *d_mask, int64_t n_rows,
                      int64_t n_chan, bool skip_zero, double *w_min,
                      double *w_max, int64_t *count, void *scratch8,
                      cudaStream_t s) {
  unsigned long long init[3] = {~0ull, 0ull, 0ull};
  unsigned long long *d = (unsigned long long *)scratch8;
  WGPU_CUDA(cudaMemcpyAsync(d, init, sizeof(init), cudaMemcpyHostToDevice, s));
  const int64_t n = n_rows * n_chan;
  unsigned blocks = (unsigned)std::min<int64_t>(grid_for(n, kThreads), (int64_t)sm_count() * 8);
  const Selector sel{skip_zero ? (const float2 *)d_vis : nullptr, d_mask};
  if (n_chan >= kExtentRowsMinChan && n_chan <= kExtentRowsMaxChan) {
    // one warp per row, two products per row
    int *rank = (int *)(d + 8);
    double *by_rank = (double *)(rank + ((n_chan + 1) & ~(int64_t)1));
    channel_rank_kernel<<<grid_for(n_chan, 128), 128, 0, s>>>(d_freq, (int)n_chan, rank, by_rank);
    check_launch("channel_rank_kernel");
    const unsigned rblocks =
        (unsigned)std::min<int64_t>((n_rows + kThreads / 8 - 1) / (kThreads / 8),
                                    (int64_t)sm_count() * 8);
    w_extent_rows_kernel<<<rblocks, kThreads, (sizeof(double) + sizeof(int)) * n_chan, s>>>(
        d_uvw, rank, by_rank, sel, n_rows, (int)n_chan, d);
  } else if (n_chan <= 4096) {
    w_extent_kernel<true><<<blocks, kThreads, sizeof(double) * n_chan, s>>>(d_uvw, d_freq, sel,
                                                                           n_rows, n_chan, d);
  } else {
    w_extent_kernel<false><<<blocks, kThreads, 0, s>>>(d_uvw, d_freq, sel, n_rows, n_chan, d);
  }
  check_launch("w_extent_kernel");
  unsigned long long out[3];
  WGPU_CUDA(cudaMemcpyAsync(out, d, sizeof(out), cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaStreamSynchronize(s));
  *count = (int64_t)out[2];
  if (out[2] == 0) {
    *w_min = *w_max = 0.0;
  } else {
    *w_min = dkey_inv(out[0]);
    *w_max = dkey_inv(out[1]);
  }
}

BucketResult bucket_visibilities(DeviceArena &arena, const DevPlan &p,
                                 const double *d_uvw, const double *d_freq,
                                 const float *d_vis, const uint8_t *d_mask,
                                 int64_t n_rows, int64_t n_chan, bool skip_zero,
                                 unsigned *wait_flags, cudaStream_t s) {
  const int64_t n = n_rows * n_chan;
  if (n >= (int64_t)0xFFFFFFFFll)
    throw Error(WGPU_ERR_INVALID, "more than 2^32-1 visibilities in one call");
  BucketResult res{};
  res.n_keys = (int64_t)p.ntu * p.ntv * 4 * p.n_planes;
  if (res.n_keys >= (int64_t)0xFFFFFFFFll)
    throw Error(WGPU_ERR_INVALID, "too many (tile, plane) buckets");
  int bits = 1;
  while (((int64_t)1 << bits) - 1 < res.n_keys) ++bits;
  const uint32_t sentinel = (uint32_t)(((uint64_t)1 << bits) - 1);

  ChannelScale *cs = (ChannelScale *)arena.get(kSlotExtent, sizeof(ChannelScale) * (n_chan + 1) + 64);
  float4 *uvwf = (float4 *)arena.get(kSlotUvwF32, sizeof(float4) * 2 * (n_rows + 1));
  float4 *uvwl = uvwf + (n_rows + 1);
  uint32_t *keys = (uint32_t *)arena.get(kSlotKeys, sizeof(uint32_t) * (n + 1));
  uint32_t *keys2 = (uint32_t *)arena.get(kSlotKeysAlt, sizeof(uint32_t) * (n + 1));
  uint32_t *vals = (uint32_t *)arena.get(kSlotVals, sizeof(uint32_t) * (n + 1));
  uint32_t *vals2 = (uint32_t *)arena.get(kSlotValsAlt, sizeof(uint32_t) * (n + 1));
  uint32_t *offsets = (uint32_t *)arena.get(kSlotOffsets, sizeof(uint32_t) * (res.n_keys + 1));
  uint8_t *minor = (uint8_t *)arena.get(kSlotCorner, (size_t)n + 16);

  const double gu = p.dl * (double)p.nu, gv = p.dm * (double)p.nv;
  channel_scales_kernel<<<grid_for(n_chan, 128), 128, 0, s>>>(d_freq, n_chan, gu, gv, cs);
  check_launch("channel_scales_kernel");
  if ((uint64_t)p.n_planes * (uint64_t)p.nv >= 0xFFFFFFFFull)
    throw Error(WGPU_ERR_INVALID, "too many (plane, row) pairs");
  res.rows.n_planes = p.n_planes;
  res.rows.nv = p.nv;
  res.rows.buf = (uint8_t *)arena.get(kSlotRowOcc, RowOccupancy{nullptr, p.n_planes, p.nv}.bytes());
  WGPU_CUDA(cudaMemsetAsync(res.rows.corners(), 0, res.rows.cells(), s));
  if (n > 0) {
    // deferred samples listed in keys2 (free until the first radix pass),
    // their count in the word after the channel scales
    uint32_t *n_pending = (uint32_t *)(cs + n_chan + 1);
    WGPU_CUDA(cudaMemsetAsync(n_pending, 0, sizeof(uint32_t), s));
    uvw_float_kernel<<<grid_for(n_rows, kThreads), kThreads, 0, s>>>(d_uvw, n_rows, uvwf,
                                                                         uvwl);
    check_launch("uvw_float_kernel");
    // no histogram here: the keys are counted after the sort, in key order
    key_kernel<<<grid_for(n, kThreads), kThreads, 0, s>>>(
        p, d_uvw, cs, Selector{skip_zero ? (const float2 *)d_vis : nullptr, d_mask},
        n_rows, n_chan, sentinel, keys, vals, nullptr, res.rows.corners(), keys2, n_pending,
        uvwf, minor);
    check_launch("key_kernel");
    key_fix_kernel<<<sm_count() * 4, kThreads, 0, s>>>(p, d_uvw, cs, n_chan, keys2, n_pending,
                                                        keys, nullptr, res.rows.corners(), minor);
    check_launch("key_fix_kernel");
  }
  build_row_occupancy(res.rows, p.support, s);

  // the number of bucketed elements (and the first sort pass's digit totals)
  const int64_t status_words = sweep_status_words(n);
  uint64_t *status = (uint64_t *)arena.get(
      kSlotHist, sizeof(uint64_t) * status_words + sizeof(uint32_t) * (sweep_counter_words() + 1));
  sweep_count(keys, minor, n, sentinel, status, s);
  uint32_t total = 0;
  WGPU_CUDA(cudaMemcpyAsync(&total, sweep_kept_word(status, n), sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaStreamSynchronize(s));
  // radix sort over the key bits in use, the unselected samples dropped
  // without a caller's flag word, expired waits are counted in the word after the counters
  unsigned *own_flag = (unsigned *)(status + status_words) + sweep_counter_words();
  if (!wait_flags) WGPU_CUDA(cudaMemsetAsync(own_flag, 0, sizeof(unsigned), s));
  uint32_t *kin = keys, *vin = vals, *kout = keys2, *vout = vals2;
  sweep_sort_kept(kin, vin, kout, vout, minor, n, total, bits, sentinel, status,
                  wait_flags ? wait_flags : own_flag, s);
  if (!wait_flags && n > 0 && total > 0) {
    unsigned expired = 0;
    WGPU_CUDA(cudaMemcpyAsync(&expired, own_flag, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    WGPU_CUDA(cudaStreamSynchronize(s));
    if (expired) throw Error(WGPU_ERR_TIMEOUT, "a bounded device wait expired (bucket sort)");
  }
  // bucket offsets: the number of elements of each key (counted on the
  // sorted keys), then their exclusive scan
  WGPU_CUDA(cudaMemsetAsync(offsets, 0, sizeof(uint32_t) * (res.n_keys + 1), s));
  if (total > 0) {
    count_sorted_keys_kernel<<<grid_for(total, kThreads), kThreads, 0, s>>>(kin, total, offsets);
    check_launch("count_sorted_keys_kernel");
  }
  exclusive_scan_u32(arena, offsets, res.n_keys + 1, s);
  res.n_out = total;
  res.perm = vin;
  res.offsets = offsets;
  res.records = (VisRecord *)arena.get(kSlotRecords, sizeof(VisRecord) * (res.n_out + 1));
  if (res.n_out > 0) {
    const bool shift = p.l_shift != 0.0 || p.m_shift != 0.0;
    const float2 *vis = skip_zero ? (const float2 *)d_vis : nullptr;
    // undecided records listed in kout (free after the sort), counts per
    // record block in vout
    const int64_t n_blocks = (res.n_out + kRecordBlock - 1) / kRecordBlock;
    (shift ? record_ff_kernel<true> : record_ff_kernel<false>)<<<(unsigned)n_blocks, kThreads,
                                                                  0, s>>>(
        p, cs, vis, n_chan, res.perm, res.n_out, res.records, uvwf, uvwl, kout, vout);
    check_launch("record_ff_kernel");
    (shift ? record_fix_kernel<true> : record_fix_kernel<false>)<<<sm_count() * 8, kThreads, 0,
                                                                    s>>>(
        p, d_uvw, cs, vis, n_chan, res.perm, n_blocks, res.records, uvwf, kout, vout);
    check_launch("record_fix_kernel");
  }
  return res;
}


// ---------------------------------------------------------------------------
// Allocation-free bucketing.
//
// Some callers cannot allocate device memory while they call this library: a
// host that owns the whole device memory through its own pool, code running
// under a memory budget that forbids new allocations, or a pipeline that must
// not trigger the device-wide synchronisation a cudaMalloc / cudaFree may
// cause.  For them the bucketing pass keeps its scratch (sort keys and values
// in two copies, per-block digit histograms, scan partial sums, channel
// scales) in the file-scope device array below, sized for at most
// kNoallocMaxVis visibilities and kNoallocMaxChan channels.  Every GPU that
// loads the library holds this array until the process exits.  Its address is
// looked up once per device (cudaGetSymbolAddress, with that device current)
// on the first call made on the device.  All calls share the array and it keeps
// the contents of the last call: calls whose work overlaps on the GPU (other
// streams, other host threads) race with each other and must be serialised by
// the caller.
// ---------------------------------------------------------------------------
namespace {
constexpr int64_t kNoallocMaxVis = WGPU_NOALLOC_MAX_VISIBILITIES;
constexpr int64_t kNoallocMaxChan = WGPU_NOALLOC_MAX_CHANNELS;
constexpr int64_t kNoallocMaxKeys = (int64_t)1 << 26;
constexpr int64_t kNoallocBlocks = (kNoallocMaxVis + kSortTile - 1) / kSortTile;
constexpr size_t kNoallocScanWords = ((kNoallocMaxKeys + 1) / 4096 + 64 + 255) / 256 * 256;
constexpr size_t kNoallocSortBytes = 4 * sizeof(uint32_t) * kNoallocMaxVis;
constexpr size_t kNoallocHistBytes = sizeof(uint32_t) * 256 * kNoallocBlocks;
constexpr size_t kNoallocScanBytes = sizeof(uint32_t) * kNoallocScanWords;
constexpr size_t kNoallocScaleBytes = (sizeof(ChannelScale) * kNoallocMaxChan + 255) / 256 * 256;
constexpr size_t kNoallocCornerBytes = (size_t)kNoallocMaxVis;
constexpr size_t kNoallocBytes = kNoallocSortBytes + kNoallocHistBytes + kNoallocScanBytes +
                                 kNoallocScaleBytes + kNoallocCornerBytes;
}  // namespace

static __device__ __align__(256) unsigned char g_bucket_scratch[kNoallocBytes];

size_t bucket_noalloc_scratch_bytes() { return kNoallocBytes; }

// Device address of g_bucket_scratch for the current device, looked up once.
static unsigned char *bucket_scratch_address() {
  static std::mutex mu;
  static unsigned char *addr[256] = {};
  int dev = 0;
  WGPU_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) throw Error(WGPU_ERR_CUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_bucket_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      throw Error(WGPU_ERR_CUDA, std::string("cudaGetSymbolAddress of the bucketing scratch: ") +
                                     cudaGetErrorString(e));
    }
    addr[dev] = (unsigned char *)p;
  }
  return addr[dev];
}

int64_t bucket_visibilities_noalloc(const DevPlan &p, const double *d_uvw, const double *d_freq,
                                    const float *d_vis, int64_t n_rows, int64_t n_chan,
                                    bool skip_zero, VisRecord *d_records, uint32_t *d_perm,
                                    uint32_t *d_offsets, cudaStream_t s) {
  const int64_t n = n_rows * n_chan;
  if (n > kNoallocMaxVis)
    throw Error(WGPU_ERR_INVALID, "allocation-free bucketing takes at most " +
                                      std::to_string(kNoallocMaxVis) + " visibilities, got " +
                                      std::to_string(n));
  if (n_chan > kNoallocMaxChan)
    throw Error(WGPU_ERR_INVALID, "allocation-free bucketing takes at most " +
                                      std::to_string(kNoallocMaxChan) + " channels");
  const int64_t n_keys = (int64_t)p.ntu * p.ntv * 4 * p.n_planes;
  if (n_keys > kNoallocMaxKeys)
    throw Error(WGPU_ERR_INVALID, "plan has too many (tile, plane) buckets for the "
                                  "allocation-free bucketing");
  int bits = 1;
  while (((int64_t)1 << bits) - 1 < n_keys) ++bits;
  const uint32_t sentinel = (uint32_t)(((uint64_t)1 << bits) - 1);

  unsigned char *base = bucket_scratch_address();
  uint32_t *keys = (uint32_t *)base;
  uint32_t *keys2 = keys + kNoallocMaxVis;
  uint32_t *vals = keys2 + kNoallocMaxVis;
  uint32_t *vals2 = vals + kNoallocMaxVis;
  uint32_t *hist = (uint32_t *)(base + kNoallocSortBytes);
  uint32_t *scan_tmp = (uint32_t *)(base + kNoallocSortBytes + kNoallocHistBytes);
  ChannelScale *cs =
      (ChannelScale *)(base + kNoallocSortBytes + kNoallocHistBytes + kNoallocScanBytes);
  uint8_t *minor = base + kNoallocSortBytes + kNoallocHistBytes + kNoallocScanBytes +
                   kNoallocScaleBytes;

  const double gu = p.dl * (double)p.nu, gv = p.dm * (double)p.nv;
  if (n_chan > 0) {
    channel_scales_kernel<<<grid_for(n_chan, 128), 128, 0, s>>>(d_freq, n_chan, gu, gv, cs);
    check_launch("channel_scales_kernel");
  }
  // the histogram accumulates into the caller's offsets: start from zero
  WGPU_CUDA(cudaMemsetAsync(d_offsets, 0, sizeof(uint32_t) * (n_keys + 1), s));
  if (n > 0) {
    // deferred samples listed in keys2, their count in vals2[0] (both free
    // until the first radix pass)
    WGPU_CUDA(cudaMemsetAsync(vals2, 0, sizeof(uint32_t), s));
    key_kernel<<<grid_for(n, kThreads), kThreads, 0, s>>>(
        p, d_uvw, cs, Selector{skip_zero ? (const float2 *)d_vis : nullptr, nullptr}, n_rows,
        n_chan, sentinel, keys, vals, d_offsets, nullptr, keys2, vals2, nullptr, minor);
    check_launch("key_kernel");
    key_fix_kernel<<<sm_count() * 4, kThreads, 0, s>>>(p, d_uvw, cs, n_chan, keys2, vals2, keys,
                                                        d_offsets, nullptr, minor);
    check_launch("key_fix_kernel");
  }
  exclusive_scan_u32_scratch(d_offsets, n_keys + 1, scan_tmp, s);
  uint32_t total = 0;
  WGPU_CUDA(cudaMemcpyAsync(&total, d_offsets + n_keys, sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, s));
  WGPU_CUDA(cudaStreamSynchronize(s));
  uint32_t *kin = keys, *vin = vals, *kout = keys2, *vout = vals2;
  radix_sort_kept(kin, vin, kout, vout, minor, n, total, bits, sentinel, hist,
                  [&](uint32_t *d, int64_t m) { exclusive_scan_u32_scratch(d, m, scan_tmp, s); },
                  s);
  if (total > 0) {
    WGPU_CUDA(cudaMemcpyAsync(d_perm, vin, sizeof(uint32_t) * total, cudaMemcpyDeviceToDevice, s));
    const bool shift = p.l_shift != 0.0 || p.m_shift != 0.0;
    (shift ? record_kernel<true> : record_kernel<false>)<<<grid_for(total, kThreads), kThreads,
                                                          0, s>>>(
        p, d_uvw, cs, skip_zero ? (const float2 *)d_vis : nullptr, n_chan, vin, total,
        d_records, nullptr);
    check_launch("record_kernel");
  }
  WGPU_CUDA(cudaStreamSynchronize(s));
  return total;
}

}  // namespace wgpu
