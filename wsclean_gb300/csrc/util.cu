// Device arena, launch accounting and a device-wide exclusive scan.
#include <atomic>
#include <map>
#include <mutex>
#include <utility>

#include "wgpu_internal.h"

namespace wgpu {

namespace {
std::atomic<uint64_t> g_launches{0};
thread_local uint64_t t_launches = 0;  // this thread's share (graph capture)
}

void count_launch(int n) {
  g_launches.fetch_add((uint64_t)n);
  t_launches += (uint64_t)n;
}
uint64_t launch_count() { return g_launches.load(); }
uint64_t thread_launch_count() { return t_launches; }

// Raises the kernel's dynamic shared-memory cap to at least `bytes`, never
// lowering it: gridders on several host threads launch the same kernels with
// different sizes, and a cap lowered by one thread would make another thread's
// launch (or graph instantiation) fail.
void ensure_dynamic_smem(const void *fn, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> caps;
  int dev = 0;
  WGPU_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  size_t &cap = caps[{dev, fn}];
  if (bytes <= cap) return;
  WGPU_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cap = bytes;
}

void check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    throw Error(WGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  count_launch();
}

DeviceArena::~DeviceArena() { release(); }

int sm_count() {
  // SM count of the current device, looked up once per device ordinal
  // (gridders run on several host threads and may use different devices)
  static std::mutex mu;
  static int count[256] = {};
  int dev = 0;
  WGPU_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) throw Error(WGPU_ERR_CUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (count[dev] == 0) {
    int v = 0;
    WGPU_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    count[dev] = v > 0 ? v : 1;
  }
  return count[dev];
}

void *DeviceArena::get(int slot, size_t bytes) {
  if (slot < 0 || slot >= kSlots) throw Error(WGPU_ERR_INVALID, "arena slot");
  if (bytes == 0) bytes = 16;
  if (size_[slot] >= bytes) return ptr_[slot];
  if (ptr_[slot]) {
    cudaFree(ptr_[slot]);
    ptr_[slot] = nullptr;
    size_[slot] = 0;
  }
  // Round up by 1/8 so that slowly growing chunks do not reallocate each call.
  size_t want = bytes + bytes / 8;
  want = (want + 255) & ~size_t(255);
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw Error(WGPU_ERR_NOMEM, "device allocation of " + std::to_string(bytes) +
                                      " bytes failed: " + cudaGetErrorString(e));
    }
    want = bytes;
  }
  ptr_[slot] = p;
  size_[slot] = want;
  return p;
}

size_t DeviceArena::total() const {
  size_t t = 0;
  for (int i = 0; i < kSlots; ++i) t += size_[i];
  return t;
}

void DeviceArena::release() {
  for (int i = 0; i < kSlots; ++i) release(i);
}

void DeviceArena::release(int slot) {
  if (slot < 0 || slot >= kSlots) return;
  if (ptr_[slot]) cudaFree(ptr_[slot]);
  ptr_[slot] = nullptr;
  size_[slot] = 0;
}

// ---------------------------------------------------------------------------
// Exclusive scan (uint32, in place).  Three phases: per-chunk sums, scan of
// the sums (recursively), per-chunk local scan plus the chunk's base.
// ---------------------------------------------------------------------------
namespace {
constexpr int kScanThreads = 256;
constexpr int kScanPerThread = 16;
constexpr int kScanChunk = kScanThreads * kScanPerThread;  // 4096

__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  const uint32_t warp_base = warp > 0 ? warp_sums[warp - 1] : 0;
  *total = warp_sums[kScanThreads / 32 - 1];
  __syncthreads();
  return warp_base + x - v;
}

// The chunk's elements as groups of four: thread t takes groups t, t + 256,
// t + 512 and t + 768 (16-byte loads, consecutive threads on consecutive
// groups); a group that runs past n is read element by element.
__device__ __forceinline__ uint4 load_group(const uint32_t *d, int64_t k, int64_t n) {
  if (k + 3 < n) return *reinterpret_cast<const uint4 *>(d + k);
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (k < n) v.x = d[k];
  if (k + 1 < n) v.y = d[k + 1];
  if (k + 2 < n) v.z = d[k + 2];
  return v;
}
__device__ __forceinline__ void store_group(uint32_t *d, int64_t k, int64_t n, uint4 v) {
  if (k + 3 < n) {
    *reinterpret_cast<uint4 *>(d + k) = v;
    return;
  }
  if (k < n) d[k] = v.x;
  if (k + 1 < n) d[k + 1] = v.y;
  if (k + 2 < n) d[k + 2] = v.z;
}
constexpr int kScanGroups = kScanPerThread / 4;  // groups of four per thread

// ALIGNED: d is 16-byte aligned (group loads); otherwise element loads.
template <bool ALIGNED>
__global__ void __launch_bounds__(kScanThreads)
    scan_chunk_sums(const uint32_t *d, int64_t n, uint32_t *sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanChunk;
  uint32_t s = 0;
  if (ALIGNED) {
    uint4 v[kScanGroups];
#pragma unroll
    for (int j = 0; j < kScanGroups; ++j)
      v[j] = load_group(d, base + 4 * (threadIdx.x + kScanThreads * j), n);
#pragma unroll
    for (int j = 0; j < kScanGroups; ++j) s += v[j].x + v[j].y + v[j].z + v[j].w;
  } else {
#pragma unroll
    for (int i = 0; i < kScanPerThread; ++i) {
      const int64_t k = base + threadIdx.x + (int64_t)kScanThreads * i;
      if (k < n) s += d[k];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  __shared__ uint32_t ws[kScanThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += ws[w];
    sums[blockIdx.x] = t;
  }
}

template <bool ALIGNED>
__global__ void __launch_bounds__(kScanThreads)
    scan_chunk_local(uint32_t *d, int64_t n, const uint32_t *bases) {
  uint32_t carry = bases ? bases[blockIdx.x] : 0u;
  if (ALIGNED) {
    // groups in chunk order g = t + 256 j: one block scan per j, carried over
    const int64_t base = (int64_t)blockIdx.x * kScanChunk;
    uint4 v[kScanGroups];
#pragma unroll
    for (int j = 0; j < kScanGroups; ++j)
      v[j] = load_group(d, base + 4 * (threadIdx.x + kScanThreads * j), n);
#pragma unroll
    for (int j = 0; j < kScanGroups; ++j) {
      uint32_t total;
      const uint32_t ex = block_exclusive_scan(v[j].x + v[j].y + v[j].z + v[j].w, &total) + carry;
      carry += total;
      const uint4 o = make_uint4(ex, ex + v[j].x, ex + v[j].x + v[j].y,
                                 ex + v[j].x + v[j].y + v[j].z);
      store_group(d, base + 4 * (threadIdx.x + kScanThreads * j), n, o);
    }
    return;
  }
  const int64_t base = (int64_t)blockIdx.x * kScanChunk +
                       (int64_t)threadIdx.x * kScanPerThread;
  uint32_t v[kScanPerThread];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanPerThread; ++i) {
    const int64_t k = base + i;
    v[i] = k < n ? d[k] : 0u;
    s += v[i];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan(s, &total) + carry;
#pragma unroll
  for (int i = 0; i < kScanPerThread; ++i) {
    const int64_t k = base + i;
    if (k < n) d[k] = run;
    run += v[i];
  }
}

void scan_level(uint32_t *d, int64_t n, uint32_t *tmp, cudaStream_t s) {
  const int64_t nb = (n + kScanChunk - 1) / kScanChunk;
  const bool aligned = ((uintptr_t)d & 15) == 0;
  if (nb <= 1) {
    (aligned ? scan_chunk_local<true> : scan_chunk_local<false>)<<<1, kScanThreads, 0, s>>>(
        d, n, nullptr);
    check_launch("scan_chunk_local");
    return;
  }
  (aligned ? scan_chunk_sums<true> : scan_chunk_sums<false>)<<<(unsigned)nb, kScanThreads, 0,
                                                                s>>>(d, n, tmp);
  check_launch("scan_chunk_sums");
  scan_level(tmp, nb, tmp + nb, s);
  (aligned ? scan_chunk_local<true> : scan_chunk_local<false>)<<<(unsigned)nb, kScanThreads, 0,
                                                                  s>>>(d, n, tmp);
  check_launch("scan_chunk_local");
}
}  // namespace

void exclusive_scan_u32(DeviceArena &arena, uint32_t *d, int64_t n,
                        cudaStream_t s) {
  if (n <= 0) return;
  int64_t need = 0, m = n;
  while (m > kScanChunk) {
    m = (m + kScanChunk - 1) / kScanChunk;
    need += m;
  }
  uint32_t *tmp = (uint32_t *)arena.get(kSlotScanTmp, sizeof(uint32_t) * (need + 16));
  scan_level(d, n, tmp, s);
}

int64_t exclusive_scan_scratch_words(int64_t n) {
  int64_t need = 0, m = n;
  while (m > kScanChunk) {
    m = (m + kScanChunk - 1) / kScanChunk;
    need += m;
  }
  return need + 16;
}

void exclusive_scan_u32_scratch(uint32_t *d, int64_t n, uint32_t *tmp, cudaStream_t s) {
  if (n <= 0) return;
  scan_level(d, n, tmp, s);
}

}  // namespace wgpu
