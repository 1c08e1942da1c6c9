// Onesweep LSD radix sort of (Morton code, triangle id) pairs.
//
// Replaces the reference's std::sort on the code (core/builders/lbvh.cpp:755)
// with a stable GPU sort (Adinets & Merrill, "Onesweep: A Faster Least
// Significant Digit Radix Sort for GPUs", 2022):
//   1. one histogram pass counts all four 8-bit digits of every key;
//   2. a one-block kernel turns the four histograms into exclusive digit bases;
//   3. four digit passes, each ONE kernel: a tile of 4096 pairs is ranked in
//      shared memory (warp-level __match_any_sync ranking, stable), the tile's
//      per-digit counts are published and the exclusive prefix over earlier
//      tiles is found by decoupled look-back, then the tile is written out
//      grouped by digit.
// Tiles are numbered in the order blocks start (atomic ticket), so every tile
// a block waits on belongs to a block that is already resident; each wait is
// still bounded and reports kErrWaitTimeout instead of spinning forever.
//
// The segmented variant sorts many geometries' pairs in one go: after the four
// code passes, one more stable pass per byte of the segment index (the digit
// of an element is looked up from its triangle id) makes the order
// segment-major while keeping each segment's code order and ties.
#include "build_common.cuh"
#include "hrt_kernels.cuh"

namespace hrt
{
namespace
{

constexpr int      kThreads    = 256;
constexpr int      kWarps      = kThreads / 32;
constexpr int      kItems      = 16;
constexpr uint32_t kTile       = kTileSize;  // 4096 pairs
static_assert(kTile == kThreads * kItems, "tile = threads x items");
constexpr int      kRadix      = 256;
constexpr int      kPasses     = 4;
constexpr uint32_t kFlagAgg    = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask  = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit  = 1u << 22;

__device__ __forceinline__ void store_relaxed(uint32_t* p, uint32_t v)
{
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t load_relaxed(const uint32_t* p)
{
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Digit of an element for one pass: a byte of the key, or - for the segment
// passes of the segmented sort - a byte of the index of the segment that holds
// the element's value (ascending offsets[0..segCount]; value = global
// triangle index).
__device__ __forceinline__ uint32_t pass_digit(uint32_t key, uint32_t val, uint32_t shift,
                                               const uint32_t* __restrict__ segOffsets, uint32_t segCount)
{
  if (segOffsets == nullptr) return (key >> shift) & 0xFFu;
  return (bc::find_segment(segOffsets, segCount, val) >> shift) & 0xFFu;
}

// Histogram of one byte of the segment index over all elements: each segment
// adds its element count to the bin of its byte.
__global__ void k_segment_histogram(const uint32_t* __restrict__ segOffsets, uint32_t segCount, uint32_t shift,
                                    uint32_t* __restrict__ hist)
{
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < segCount; s += gridDim.x * blockDim.x)
  {
    const uint32_t c = segOffsets[s + 1] - segOffsets[s];
    if (c) atomicAdd(&hist[(s >> shift) & 0xFFu], c);
  }
}

__global__ void __launch_bounds__(kThreads) k_histogram(const uint32_t* __restrict__ keys, uint32_t n,
                                                        uint32_t* __restrict__ hist)
{
  __shared__ uint32_t sh[kPasses * kRadix];
  for (int i = threadIdx.x; i < kPasses * kRadix; i += kThreads) sh[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
  {
    const uint32_t k = keys[i];
#pragma unroll
    for (int p = 0; p < kPasses; p++) atomicAdd(&sh[p * kRadix + ((k >> (8 * p)) & 0xFF)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kPasses * kRadix; i += kThreads)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// Exclusive scan of a value held by each of the 256 threads; returns the
// exclusive prefix, *total receives the sum.  Uses `warpSums` (8 entries).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warpSums, uint32_t* total)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warpSums[warp] = incl;
  __syncthreads();
  if (warp == 0)
  {
    uint32_t w = (lane < kWarps) ? warpSums[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < kWarps) warpSums[lane] = wi - w;  // exclusive per warp
    if (lane == kWarps - 1) warpSums[kWarps] = wi;
  }
  __syncthreads();
  const uint32_t r = incl - v + warpSums[warp];
  *total = warpSums[kWarps];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kThreads) k_scan_histograms(uint32_t* __restrict__ hist, int nHist)
{
  __shared__ uint32_t warpSums[kWarps + 1];
  for (int p = 0; p < nHist; p++)
  {
    uint32_t total;
    const uint32_t v = hist[p * kRadix + threadIdx.x];
    const uint32_t e = block_exclusive_scan(v, warpSums, &total);
    hist[p * kRadix + threadIdx.x] = e;
  }
}

__global__ void __launch_bounds__(kThreads, 4) k_onesweep(const uint32_t* __restrict__ keysIn,
                                                       const uint32_t* __restrict__ valsIn,
                                                       uint32_t* __restrict__ keysOut, uint32_t* __restrict__ valsOut,
                                                       uint32_t n, uint32_t shift, const uint32_t* __restrict__ digitBase,
                                                       uint32_t* tileStatus, uint32_t* tileCounter, uint32_t* errorWord,
                                                       const uint32_t* __restrict__ segOffsets, uint32_t segCount)
{
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warpHist[kWarps][kRadix];  // counts, then per-warp exclusive offsets
  __shared__ uint32_t s_digitStart[kRadix];        // tile-local start of each digit
  __shared__ uint32_t s_dst[kRadix];               // global position = s_dst[d] + tile-local position
  __shared__ uint32_t s_warpSums[kWarps + 1];
  __shared__ uint32_t s_keys[kTile];
  __shared__ uint32_t s_vals[kTile];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(tileCounter, 1u);
  for (int i = tid; i < kWarps * kRadix; i += kThreads) (&s_warpHist[0][0])[i] = 0u;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t tileBase = tile * kTile;
  const uint32_t warpBase = tileBase + warp * (kItems * 32);

  // Warp-striped load: item k of lane l is element warpBase + 32k + l, so the
  // (warp, k, lane) order is the input order and the ranking below is stable.
  uint32_t key[kItems], val[kItems], rank[kItems];
#pragma unroll
  for (int k = 0; k < kItems; k++)
  {
    const uint32_t i = warpBase + k * 32 + lane;
    const bool valid = i < n;
    key[k] = valid ? keysIn[i] : 0xFFFFFFFFu;
    val[k] = valid ? valsIn[i] : 0u;
  }
  const uint32_t ltMask = (1u << lane) - 1u;
#pragma unroll
  for (int k = 0; k < kItems; k++)
  {
    const bool valid = (warpBase + k * 32 + lane) < n;
    const uint32_t digit = valid ? pass_digit(key[k], val[k], shift, segOffsets, segCount) : 0xFFu;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, valid ? digit : (0x100u + lane));
    const uint32_t before = s_warpHist[warp][digit];
    rank[k] = before + __popc(peers & ltMask);
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) s_warpHist[warp][digit] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Thread d owns digit d: per-warp offsets, tile total, publish, look back.
  const uint32_t d = tid;
  uint32_t total = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++)
  {
    const uint32_t c = s_warpHist[w][d];
    s_warpHist[w][d] = total;
    total += c;
  }
  uint32_t* myStatus = tileStatus + (size_t)tile * kRadix + d;
  store_relaxed(myStatus, (tile == 0 ? kFlagPrefix : kFlagAgg) | total);
  uint32_t blockTotal;
  s_digitStart[d] = block_exclusive_scan(total, s_warpSums, &blockTotal);

  uint32_t excl = 0;
  if (tile > 0)
  {
    int64_t t = (int64_t)tile - 1;
    uint32_t spins = 0;
    while (t >= 0)
    {
      const uint32_t s = load_relaxed(tileStatus + (size_t)t * kRadix + d);
      const uint32_t flag = s & ~kValueMask;
      if (flag == 0u)
      {
        if (++spins > kSpinLimit)
        {
          atomicOr(errorWord, kErrWaitTimeout);
          break;
        }
        if (spins > 64) __nanosleep(32);
        continue;
      }
      excl += s & kValueMask;
      if (flag == kFlagPrefix) break;
      t--;
    }
    store_relaxed(myStatus, kFlagPrefix | (excl + total));
  }
  s_dst[d] = digitBase[d] + excl - s_digitStart[d];
  __syncthreads();

#pragma unroll
  for (int k = 0; k < kItems; k++)
  {
    if ((warpBase + k * 32 + lane) < n)
    {
      const uint32_t digit = pass_digit(key[k], val[k], shift, segOffsets, segCount);
      const uint32_t pos = s_digitStart[digit] + s_warpHist[warp][digit] + rank[k];
      s_keys[pos] = key[k];
      s_vals[pos] = val[k];
    }
  }
  __syncthreads();

  const uint32_t count = (n - tileBase < kTile) ? (n - tileBase) : kTile;
  for (uint32_t i = tid; i < count; i += kThreads)
  {
    const uint32_t k = s_keys[i];
    const uint32_t dst = s_dst[pass_digit(k, s_vals[i], shift, segOffsets, segCount)] + i;
    if (dst < n)  // always true unless a look-back wait gave up (reported through errorWord)
    {
      keysOut[dst] = k;
      valsOut[dst] = s_vals[i];
    }
  }
}

}  // namespace

// Scratch of a four-pass sort of n pairs: digit histograms, pass counters,
// and one look-back status word per tile and digit for every pass.
constexpr size_t sort_scratch_bytes(size_t n)
{
  return sizeof(uint32_t) *
         (kPasses * kRadix + kPasses + 4 + (size_t)kPasses * ((n + kTile - 1) / kTile) * kRadix);
}

size_t radix_sort_scratch_bytes(uint32_t n) { return sort_scratch_bytes(n); }

cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keysAlt, uint32_t* valsAlt, uint32_t n,
                             void* scratch, uint32_t* errorWord, int numSMs, cudaStream_t stream)
{
  if (n <= 1) return cudaSuccess;
  const uint32_t tiles = (n + kTile - 1) / kTile;
  uint32_t* hist = (uint32_t*)scratch;
  uint32_t* counters = hist + kPasses * kRadix;
  uint32_t* status = counters + kPasses + 4;
  cudaError_t e = cudaMemsetAsync(scratch, 0, radix_sort_scratch_bytes(n), stream);
  if (e != cudaSuccess) return e;
  uint32_t hb = (n + kThreads - 1) / kThreads;
  const uint32_t maxHb = (uint32_t)numSMs * 4u;
  if (hb > maxHb) hb = maxHb;
  k_histogram<<<hb, kThreads, 0, stream>>>(keys, n, hist);
  k_scan_histograms<<<1, kThreads, 0, stream>>>(hist, kPasses);
  uint32_t* srcK = keys;
  uint32_t* srcV = vals;
  uint32_t* dstK = keysAlt;
  uint32_t* dstV = valsAlt;
  for (int p = 0; p < kPasses; p++)
  {
    k_onesweep<<<tiles, kThreads, 0, stream>>>(srcK, srcV, dstK, dstV, n, 8u * p, hist + p * kRadix,
                                               status + (size_t)p * tiles * kRadix, counters + p, errorWord, nullptr, 0u);
    uint32_t* t = srcK; srcK = dstK; dstK = t;
    t = srcV; srcV = dstV; dstV = t;
  }
  return cudaGetLastError();  // four passes: the result is back in keys/vals
}

// Number of segment-index bytes the segmented sort passes over.
static int segment_passes(uint32_t segCount)
{
  int p = 1;
  while (p < 4 && (segCount - 1u) >> (8 * p)) p++;
  return p;
}

size_t radix_sort_segmented_scratch_bytes(uint32_t n, uint32_t segCount)
{
  const size_t tiles = (n + kTile - 1) / kTile;
  const size_t passes = kPasses + segment_passes(segCount);
  return sizeof(uint32_t) * (passes * kRadix + passes + 4 + passes * tiles * kRadix);
}

cudaError_t radix_sort_pairs_segmented(uint32_t* keys, uint32_t* vals, uint32_t* keysAlt, uint32_t* valsAlt,
                                       uint32_t n, const uint32_t* segOffsets, uint32_t segCount, void* scratch,
                                       uint32_t* errorWord, int numSMs, cudaStream_t stream)
{
  if (n <= 1) return cudaSuccess;
  const int segPasses = segment_passes(segCount);
  const int passes = kPasses + segPasses;
  const uint32_t tiles = (n + kTile - 1) / kTile;
  uint32_t* hist = (uint32_t*)scratch;
  uint32_t* counters = hist + passes * kRadix;
  uint32_t* status = counters + passes + 4;
  cudaError_t e = cudaMemsetAsync(scratch, 0, radix_sort_segmented_scratch_bytes(n, segCount), stream);
  if (e != cudaSuccess) return e;
  uint32_t hb = (n + kThreads - 1) / kThreads;
  const uint32_t maxHb = (uint32_t)numSMs * 4u;
  if (hb > maxHb) hb = maxHb;
  k_histogram<<<hb, kThreads, 0, stream>>>(keys, n, hist);
  for (int q = 0; q < segPasses; q++)
    k_segment_histogram<<<(segCount + 255) / 256, 256, 0, stream>>>(segOffsets, segCount, 8u * q,
                                                                     hist + (kPasses + q) * kRadix);
  k_scan_histograms<<<1, kThreads, 0, stream>>>(hist, passes);
  uint32_t* srcK = keys;
  uint32_t* srcV = vals;
  uint32_t* dstK = keysAlt;
  uint32_t* dstV = valsAlt;
  // code bytes first (least significant), then the segment index bytes: a
  // stable LSD sort by (segment, code) keeps the input order among ties
  for (int p = 0; p < passes; p++)
  {
    const bool seg = p >= kPasses;
    k_onesweep<<<tiles, kThreads, 0, stream>>>(srcK, srcV, dstK, dstV, n, seg ? 8u * (p - kPasses) : 8u * p,
                                               hist + p * kRadix, status + (size_t)p * tiles * kRadix, counters + p,
                                               errorWord, seg ? segOffsets : nullptr, segCount);
    uint32_t* t = srcK; srcK = dstK; dstK = t;
    t = srcV; srcV = dstV; dstV = t;
  }
  if (srcK != keys)
  {
    e = cudaMemcpyAsync(keys, srcK, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, stream);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(vals, srcV, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, stream);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace hrt

// ---------------------------------------------------------------------------
// Allocation-free variant of the pair sort (hrt_sort_morton_pairs_noalloc).
//
// Some callers cannot call cudaMalloc: host applications whose device memory
// is owned by another allocator that reserves it up front (a renderer or a
// game engine with its own heap, a process under a hard device-memory quota),
// and latency-bound paths that cannot afford the implicit synchronisation of
// an allocation.  For them this entry point takes its scratch (ping-pong
// arrays, digit histograms, look-back tile status and an error word) from one
// file-scope device array of fixed size, so it calls no allocator at all.
// The array is part of the library image: every GPU that loads the library
// holds kNoAllocScratchBytes of it until the process exits.
#include <mutex>

#include "../../include/hrt.h"

namespace
{

constexpr uint32_t kNoAllocMaxPairs  = HRT_NOALLOC_MAX_PAIRS;
constexpr uint32_t kNoAllocTiles     = (kNoAllocMaxPairs + hrt::kTileSize - 1) / hrt::kTileSize;
constexpr size_t   kNoAllocSortBytes = hrt::sort_scratch_bytes(kNoAllocMaxPairs);
static_assert(kNoAllocSortBytes == sizeof(uint32_t) * (4 * 256 + 4 + 4 + (size_t)4 * kNoAllocTiles * 256),
              "the fixed array holds the scratch of a sort of HRT_NOALLOC_MAX_PAIRS pairs");
constexpr size_t   kNoAllocPingPong  = sizeof(uint32_t) * (size_t)kNoAllocMaxPairs;  // one array
constexpr size_t   kNoAllocScratchBytes = 2 * kNoAllocPingPong + kNoAllocSortBytes + 256;
constexpr int      kNoAllocMaxDevices = 64;

// Scratch shared by every call on a device; in host code this name is only a
// stand-in, the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

std::mutex g_noallocMu;
void*      g_noallocPtr[kNoAllocMaxDevices] = {};
int        g_noallocSMs[kNoAllocMaxDevices] = {};

}  // namespace

extern "C" int hrt_sort_morton_pairs_noalloc(uint32_t* keys, uint32_t* vals, uint64_t n, void* stream)
{
  if (n > kNoAllocMaxPairs) return HRT_ERR_CAPACITY;
  if (n > 0 && (!keys || !vals)) return HRT_ERR_INVALID_ARGUMENT;
  if (n <= 1) return HRT_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return HRT_ERR_CUDA;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return HRT_ERR_UNSUPPORTED;
  void* base = nullptr;
  int numSMs = 0;
  {
    // One-time set-up per device, with that device current: resolve the
    // device address of the scratch array.  The address is kept for the life
    // of the process, so the entry point must not be used on a device after
    // cudaDeviceReset (or any other teardown of its primary context).
    std::lock_guard<std::mutex> lk(g_noallocMu);
    if (!g_noallocPtr[dev])
    {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noallocScratch) != cudaSuccess || !p) return HRT_ERR_CUDA;
      int sms = 0;
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return HRT_ERR_CUDA;
      g_noallocSMs[dev] = sms;
      g_noallocPtr[dev] = p;
    }
    base = g_noallocPtr[dev];
    numSMs = g_noallocSMs[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* b = (unsigned char*)base;
  uint32_t* keysAlt = (uint32_t*)b;
  uint32_t* valsAlt = (uint32_t*)(b + kNoAllocPingPong);
  void* sortScratch = b + 2 * kNoAllocPingPong;
  uint32_t* errorWord = (uint32_t*)(b + 2 * kNoAllocPingPong + kNoAllocSortBytes);
  // The array keeps the previous call's contents: clear what must start at zero.
  if (cudaMemsetAsync(errorWord, 0, sizeof(uint32_t), s) != cudaSuccess) return HRT_ERR_CUDA;
  if (hrt::radix_sort_pairs(keys, vals, keysAlt, valsAlt, (uint32_t)n, sortScratch, errorWord, numSMs, s) != cudaSuccess)
    return HRT_ERR_CUDA;
  uint32_t err = 0;
  if (cudaMemcpyAsync(&err, errorWord, sizeof(err), cudaMemcpyDeviceToHost, s) != cudaSuccess) return HRT_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return HRT_ERR_CUDA;
  return (err & hrt::kErrWaitTimeout) ? HRT_ERR_TIMEOUT : HRT_OK;
}
