// Device helpers shared by the single-geometry build (build.cu) and the
// segmented multi-geometry build (build_batch.cu).
#pragma once

#include "hrt_common.cuh"

namespace hrt
{
namespace bc
{

constexpr int      kScanItems  = 16;    // items per thread of the look-back scans
constexpr uint32_t kFlagAgg    = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask  = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit  = 1u << 22;  // bounded look-back wait

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

__device__ __forceinline__ uint32_t atomic_add_acq_rel(uint32_t* p, uint32_t v)
{
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// A node written by other threads of the same kernel, read through L2 in two
// 16-byte loads: {boxMin, leftOffset}, {boxMax, escapeIndex}.
__device__ __forceinline__ void load_node_cg(const BVHNode32* n, float4& lo, float4& hi)
{
  const float4* p = reinterpret_cast<const float4*>(n);
  lo = __ldcg(p);
  hi = __ldcg(p + 1);
}

// Parent box from its children's (lm_min / lm_max per axis), stored with the
// child links in two 16-byte stores.
__device__ __forceinline__ void store_parent(BVHNode32* n, const float4& alo, const float4& ahi, const float4& blo,
                                             const float4& bhi, uint32_t l, uint32_t r)
{
  float4* p = reinterpret_cast<float4*>(n);
  p[0] = make_float4(lm_min(alo.x, blo.x), lm_min(alo.y, blo.y), lm_min(alo.z, blo.z), __uint_as_float(l));
  p[1] = make_float4(lm_max(ahi.x, bhi.x), lm_max(ahi.y, bhi.y), lm_max(ahi.z, bhi.z), __uint_as_float(r));
}

// SpreadBits / ZIndex3D, core/builders/lbvh.cpp:25-39.
__device__ __forceinline__ uint32_t spread_bits(int x, int offset)
{
  x = (x | (x << 10)) & 0x000F801F;
  x = (x | (x << 4)) & 0x00E181C3;
  x = (x | (x << 2)) & 0x03248649;
  x = (x | (x << 2)) & 0x09249249;
  return (uint32_t)x << offset;
}

// Morton code of one triangle (kernel1D_EvalMortonCodesFromTriangles,
// core/builders/lbvh.cpp:259-287): box centre, or the centroid
// 0.33333333*(v1+v2+v3) when the geometry has fewer than 256 triangles,
// quantised against the scene box with truncation toward zero.
__device__ __forceinline__ uint32_t morton_code(const float4& a, const float4& b, const float4& c, uint32_t nTris,
                                                const float* bmin, const float* scale)
{
  const float pa[3] = {a.x, a.y, a.z}, pb[3] = {b.x, b.y, b.z}, pc[3] = {c.x, c.y, c.z};
  int q[3];
#pragma unroll
  for (int k = 0; k < 3; k++)
  {
    float center;
    if (nTris < 256)
      center = __fmul_rn(0.33333333f, __fadd_rn(__fadd_rn(pa[k], pb[k]), pc[k]));
    else
    {
      const float mn = lm_min(pa[k], lm_min(pb[k], pc[k]));
      const float mx = lm_max(pa[k], lm_max(pb[k], pc[k]));
      center = __fmul_rn(__fadd_rn(mn, mx), 0.5f);
    }
    q[k] = __float2int_rz(__fmul_rn(scale[k], __fsub_rn(center, bmin[k])));
  }
  return spread_bits(q[0], 0) | spread_bits(q[1], 1) | spread_bits(q[2], 2);
}

// ZIndexMultCoeff on the box widened by 1e-4 (core/builders/lbvh.cpp:41-51,263).
// cubic = 1 (the engine's HRT_MORTON_CUBIC frame, no reference counterpart):
// x, y and z share the scale of the longest widened extent, so a cell of the
// Morton grid is a cube and a flat scene (a heightfield) does not spend a
// third of the code's bits splitting its thin axis; the codes are still
// 3 x 10 bits in [0, 1023] per axis.
__device__ __forceinline__ void zindex_scale(const float* mn, const float* mx, BuildParams* params, int cubic = 0)
{
  float ext[4];
  for (int c = 0; c < 4; c++)
  {
    params->bmin[c] = mn[c];
    params->bmax[c] = mx[c];
    const float lo = __fsub_rn(mn[c], 1e-4f);
    const float hi = __fadd_rn(mx[c], 1e-4f);
    ext[c] = __fsub_rn(hi, lo);
  }
  const float emax = lm_max(ext[0], lm_max(ext[1], ext[2]));
  for (int c = 0; c < 4; c++)
  {
    const float e = (cubic && c < 3) ? emax : ext[c];
    float inv = __fdiv_rn(1.0f, e);
    if (c < 3 && fabsf(e) < 1e-20f) inv = 0.0f;
    params->scale[c] = __fmul_rn(1024.0f, inv);
  }
}

// delta() of core/builders/lbvh.cpp:386-403 against a code held in a
// register: the codes are unique after compaction, so this is the count of
// leading zeros of their XOR (32 for equal codes, -1 out of range).
__device__ __forceinline__ int karras_delta(const uint32_t* __restrict__ c, int L, uint32_t ci, int j)
{
  if (j < 0 || j >= L) return -1;
  const uint32_t x = ci ^ __ldg(c + j);
  return x == 0u ? 32 : __clz(x);
}

__device__ __forceinline__ int clz_delta(uint32_t a, uint32_t b)
{
  const uint32_t x = a ^ b;
  return x == 0u ? 32 : __clz(x);
}

// Node i's code and its neighbours' deltas, exchanged across the warp: lane l
// handles absolute code index g (-1: no node); the neighbours' codes come
// from the adjacent lanes by __shfl_up_sync / __shfl_down_sync when those
// lanes hold indices g - 1 and g + 1 of the same tree, from memory otherwise
// (the warp's first and last lanes, tree boundaries of a segmented build).
// Every lane of the warp must call this.
__device__ __forceinline__ void karras_neighbours(const uint32_t* __restrict__ all, int segBase, int L, int i,
                                                  bool active, uint32_t& ci, int& dPrev, int& dNext)
{
  const int g = active ? segBase + i : -1;
  ci = active ? __ldg(all + g) : 0u;
  const uint32_t up = __shfl_up_sync(0xFFFFFFFFu, ci, 1);
  const int gUp = __shfl_up_sync(0xFFFFFFFFu, g, 1);
  const uint32_t down = __shfl_down_sync(0xFFFFFFFFu, ci, 1);
  const int gDown = __shfl_down_sync(0xFFFFFFFFu, g, 1);
  const int lane = (int)(threadIdx.x & 31u);
  dPrev = -1;
  dNext = -1;
  if (!active) return;
  if (i >= 1) dPrev = clz_delta(ci, (lane > 0 && gUp == g - 1) ? up : __ldg(all + g - 1));
  if (i + 1 < L) dNext = clz_delta(ci, (lane < 31 && gDown == g + 1) ? down : __ldg(all + g + 1));
}

// kernel1D_Karras12 (core/builders/lbvh.cpp:405-441) for internal node i of a
// tree over L unique codes c (ci = c[i], dPrev / dNext = its deltas to the
// codes before and after it): direction from the neighbours' deltas, the
// range end by exponential then binary search, the split by binary search;
// children in the LR numbering (internal 0..L-2, leaves L-1..2L-2), `other` =
// the far end of the node's leaf range.
__device__ __forceinline__ void karras_node(const uint32_t* __restrict__ c, int L, int i, uint32_t ci, int dPrev,
                                            int dNext, uint32_t& left, uint32_t& right, int& other)
{
  const int dl = dNext - dPrev;
  const int d = (dl > 0) - (dl < 0);
  const int dmin = d > 0 ? dPrev : (d < 0 ? dNext : 32);  // delta(i, i - d)
  int lmax = 2;
  while (karras_delta(c, L, ci, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t > 0; t >>= 1)
    if (karras_delta(c, L, ci, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = karras_delta(c, L, ci, j);
  int s = 0;
  for (int t = (l + 1) >> 1; t > 0; t = (t == 1 ? 0 : (t + 1) >> 1))
    if (karras_delta(c, L, ci, i + (s + t) * d) > dnode) s += t;
  const int gamma = i + s * d + (d < 0 ? d : 0);
  left = ((i < j ? i : j) == gamma) ? (uint32_t)(L - 1 + gamma) : (uint32_t)gamma;
  right = ((i > j ? i : j) == gamma + 1) ? (uint32_t)(L - 1 + gamma + 1) : (uint32_t)(gamma + 1);
  other = j;
}

// Leaves per block of the bottom-up refit: the nodes whose leaf range lies in
// a block's slice finish with counters in shared memory.
constexpr uint32_t kRefitSlice = 512;
// One refit thread per leaf of the slice, so a slice's walks run side by side,
// at 32 registers so that four blocks (64 warps) fit on an SM: the walks are
// chains of dependent loads and atomics, and the warps in flight hide them.
constexpr int kRefitThreads = 512;
constexpr int kRefitMinBlocks = 4;

__device__ __forceinline__ uint32_t atomic_add_acq_rel_cta(uint32_t* p, uint32_t v)
{
  uint32_t old;
  asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], %2;"
               : "=r"(old)
               : "r"((uint32_t)__cvta_generic_to_shared(p)), "r"(v)
               : "memory");
  return old;
}

// Index of the segment containing position x: the largest s with
// offsets[s] <= x, for ascending offsets[0..count] (offsets[0] = 0).
__device__ __forceinline__ uint32_t find_segment(const uint32_t* __restrict__ offsets, uint32_t count, uint32_t x)
{
  uint32_t lo = 0, hi = count;  // answer in [lo, hi)
  while (hi - lo > 1)
  {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(offsets + mid) <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// One tile (THREADS x kScanItems codes) of the run compaction
// (kernel1D_AppendInit + exclusive_scan + kernel1D_AppendComplete,
// core/builders/lbvh.cpp:289-319,762-767) as a single-pass scan with decoupled
// look-back: a position starts a run when its code differs from its
// predecessor's or (segmented build) when it starts a segment; run starts are
// appended to (compressed, runStarts) in order and the last tile writes the
// run count to *total.
template <int THREADS>
__device__ __forceinline__ void compact_runs_tile(const uint32_t* __restrict__ keys, uint32_t n,
                                                  const uint32_t* __restrict__ segOffsets, uint32_t segCount,
                                                  uint32_t* __restrict__ compressed, uint32_t* __restrict__ runStarts,
                                                  uint32_t* tileStatus, uint32_t* tileCounter, uint32_t* total,
                                                  uint32_t* errorWord)
{
  __shared__ uint32_t s_tile, s_prefix;
  __shared__ uint32_t s_warp[THREADS / 32 + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(tileCounter, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t base = tile * (THREADS * kScanItems) + tid * kScanItems;

  uint32_t key[kScanItems];
  uint32_t flags = 0, cnt = 0;
  uint32_t prev = (base > 0 && base - 1 < n) ? keys[base - 1] : 0u;
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
  {
    const uint32_t i = base + k;
    key[k] = (i < n) ? keys[i] : 0u;
    bool f = (i < n) && (i == 0 || key[k] != prev);
    if (segOffsets != nullptr && i < n && !f)
    {
      const uint32_t s = find_segment(segOffsets, segCount, i);
      f = (segOffsets[s] == i);
    }
    prev = key[k];
    flags |= (f ? 1u : 0u) << k;
    cnt += f ? 1u : 0u;
  }
  // block exclusive scan of cnt
  uint32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (tid == 0)
  {
    uint32_t run = 0;
    for (int w = 0; w < THREADS / 32; w++)
    {
      const uint32_t t = s_warp[w];
      s_warp[w] = run;
      run += t;
    }
    s_warp[THREADS / 32] = run;
    // publish and look back (one value per tile)
    uint32_t* my = tileStatus + tile;
    uint32_t excl = 0;
    if (tile == 0)
      store_relaxed(my, kFlagPrefix | run);
    else
    {
      store_relaxed(my, kFlagAgg | run);
      int64_t t = (int64_t)tile - 1;
      uint32_t spins = 0;
      while (t >= 0)
      {
        const uint32_t s = load_relaxed(tileStatus + t);
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
      store_relaxed(my, kFlagPrefix | (excl + run));
    }
    s_prefix = excl;
    const uint32_t tiles = (n + (THREADS * kScanItems) - 1) / (THREADS * kScanItems);
    if (tile == tiles - 1) *total = (excl + run <= n) ? excl + run : n;
  }
  __syncthreads();
  uint32_t pos = s_prefix + s_warp[warp] + incl - cnt;
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
    if (flags & (1u << k))
    {
      if (pos < n)  // always true unless a look-back wait gave up (reported through errorWord)
      {
        compressed[pos] = key[k];
        runStarts[pos] = base + k;
      }
      pos++;
    }
}

}  // namespace bc
}  // namespace hrt
