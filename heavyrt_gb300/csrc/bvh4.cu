// Collapse of the LBVH (binary Karras tree) into 4-wide nodes, stored as FP32
// boxes, FP16 boxes rounded outward, or 8-bit offsets against a per-node FP32
// frame with power-of-two scales (also rounded outward).
//
// Collapse rule (HeavyRT's BVH2ToBVH4, core/builders/cbvh.cpp:226-311): a
// 4-wide node replaces a binary node and its two children; its slots are the
// grandchildren (or the child itself when that child is a leaf).  A binary
// node that would become a 4-wide node while both its children are leaves is
// instead merged into one leaf covering both runs (their sorted ranges are
// adjacent).  The root always stays a node.  With this rule the 4-wide nodes
// are exactly the binary internal nodes at even depth that are not merged.
//
// Largest-first rule (a build option): a 4-wide node starts from its binary
// node's two children and twice opens the internal slot with the most leaves
// under it (the leftmost of equals) into that slot's two children, in place.
// The slots' shapes alone decide, so a refit (same topology) keeps the tree.
// Which binary nodes become 4-wide nodes then depends on the choices above
// them: the roles are found top down, one 4-wide level per launch, each level
// a frontier list built with atomics (the roles do not depend on the order
// within a level; the numbering is the same Karras-order scan as before).
//
// Quantised boxes only ever contain the FP32 box they stand for, so a
// traversal of the quantised tree visits every node the FP32 tree would and
// can only add visits; the triangle test is unchanged.
#include <cuda_fp16.h>

#include "build_common.cuh"
#include "hrt_kernels.cuh"

namespace hrt
{
namespace
{

constexpr int kThreads = 256;

// Depth of internal node i of one tree: walk up the parent chain (depth <= 30).
__device__ __forceinline__ uint8_t node_depth(const uint32_t* __restrict__ parent, uint32_t L, uint32_t i)
{
  uint32_t d = 0, n = i;
  while (n != 0 && d < 255)
  {
    const uint32_t p = parent[n];
    if (p + 1u >= L) break;  // only the root lacks an internal parent
    n = p;
    d++;
  }
  return (uint8_t)d;
}

__global__ void __launch_bounds__(kThreads) k_depth(const BuildParams* __restrict__ params,
                                                    const uint32_t* __restrict__ parent, uint8_t* __restrict__ depth)
{
  const uint32_t L = params->nLeaves;
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i + 1 < L; i += gridDim.x * kThreads)
    depth[i] = node_depth(parent, L, i);
}

// First sorted triangle and one-past-last of the triangles under binary node s.
__device__ __forceinline__ void node_range(const BVHNode32* __restrict__ lr, const uint32_t* __restrict__ runStarts,
                                           uint32_t L, uint32_t nTris, uint32_t s, uint32_t& start, uint32_t& end)
{
  // leftmost / rightmost leaf under s: follow left (right) children down
  uint32_t a = s, b = s;
  while (a + 1u < L) a = lr[a].leftOffset;
  while (b + 1u < L) b = lr[b].escapeIndex;
  const uint32_t la = a - (L - 1), lb = b - (L - 1);
  start = runStarts[la];
  end = (lb + 1 < L) ? runStarts[lb + 1] : nTris;
}

// Whether internal node i, due to become a 4-wide node, becomes one leaf instead.
// mergeMode 0: merge when both children are leaves (the reference's rule);
// mergeMode M > 0: merge when the subtree holds at most M triangles.
__device__ __forceinline__ bool merges(const BVHNode32* __restrict__ lr, const uint32_t* __restrict__ runStarts,
                                       uint32_t L, uint32_t nTris, int mergeMode, uint32_t i)
{
  if (i == 0) return false;  // the root stays a node
  if (mergeMode == 0) return lr[i].leftOffset + 1u >= L && lr[i].escapeIndex + 1u >= L;
  if (mergeMode == 1) return false;  // an internal node holds two leaves at least, so two triangles
  uint32_t st, en;
  node_range(lr, runStarts, L, nTris, i, st, en);
  return en - st <= (uint32_t)mergeMode;
}

// Role of internal node i under the even-depth rule: 1 = 4-wide node, 2 =
// merged leaf, 0 = absorbed.
__device__ __forceinline__ uint8_t node_role(const BVHNode32* __restrict__ lr, const uint32_t* __restrict__ runStarts,
                                             uint32_t L, uint32_t nTris, uint8_t depth, int mergeMode, uint32_t i)
{
  if ((depth & 1u) != 0u) return 0;
  return merges(lr, runStarts, L, nTris, mergeMode, i) ? 2 : 1;
}

constexpr int kCollapseLargestFirst = 1;  // HRT_BVH4_COLLAPSE_LARGEST_FIRST

// The binary nodes that become the slots of the 4-wide node of internal node
// i (L >= 2), left to right; returns their count (2..4).  Even depth: each
// child's two children, or the child itself when it is a leaf.  Largest
// first: the two children, then twice the internal slot with the largest
// descendant count (most leaves; the leftmost of equals) replaced in place by
// its two children.
__device__ __forceinline__ int collapse_slots(const BVHNode32* __restrict__ lr, const uint32_t* __restrict__ lrCount,
                                              uint32_t L, int collapse, uint32_t i, uint32_t (&cand)[4])
{
  const uint32_t k0 = lr[i].leftOffset, k1 = lr[i].escapeIndex;
  if (collapse != kCollapseLargestFirst)
  {
    const bool in0 = k0 + 1u < L, in1 = k1 + 1u < L;
    const uint32_t a0 = in0 ? lr[k0].leftOffset : k0, b0 = in0 ? lr[k0].escapeIndex : 0u;
    const uint32_t a1 = in1 ? lr[k1].leftOffset : k1, b1 = in1 ? lr[k1].escapeIndex : 0u;
    cand[0] = a0;
    cand[1] = in0 ? b0 : a1;
    cand[2] = in0 ? a1 : b1;
    cand[3] = b1;
    return (in0 ? 2 : 1) + (in1 ? 2 : 1);
  }
  cand[0] = k0;
  cand[1] = k1;
  cand[2] = cand[3] = 0u;
  int n = 2;
#pragma unroll
  for (int it = 0; it < 2; it++)
  {
    int best = -1;
    uint32_t bestCount = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (k < n && cand[k] + 1u < L)
      {
        const uint32_t c = lrCount[cand[k]];
        if (best < 0 || c > bestCount)
        {
          best = k;
          bestCount = c;
        }
      }
    if (best < 0) break;
    uint32_t x = 0;
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (k == best) x = cand[k];
    const uint32_t left = lr[x].leftOffset, right = lr[x].escapeIndex;
    // slots after `best` move one place right; `best` becomes the two children
#pragma unroll
    for (int k = 3; k >= 1; k--)
      if (k >= best + 2 && k <= n) cand[k] = cand[k - 1];
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
      if (k == best) cand[k] = left;
      if (k == best + 1) cand[k] = right;
    }
    n++;
  }
  return n;
}

// Appends each lane's `cnt` entries (up to four, in `item`) to a list with one
// atomic per warp; all 32 lanes call it together.  Entries at or past `cap`
// are dropped and reported.
__device__ __forceinline__ void warp_append(const uint32_t (&item)[4], int cnt, uint32_t* __restrict__ list,
                                            uint32_t* count, uint32_t cap, uint32_t* errorWord)
{
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t incl = (uint32_t)cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  uint32_t base = 0;
  if (lane == 31 && total) base = atomicAdd(count, total);
  base = __shfl_sync(0xFFFFFFFFu, base, 31) + incl - (uint32_t)cnt;
#pragma unroll
  for (int k = 0; k < 4; k++)
    if (k < cnt)
    {
      if (base + k < cap)
        list[base + k] = item[k];
      else
        atomicOr(errorWord, kErrLayout);
    }
}

// One level of the largest-first roles: every 4-wide node of this level
// (frontIn) marks its internal slots as 4-wide nodes (appended to frontOut)
// or merged leaves.  role is zeroed beforehand and the root marked.  The
// loop runs over warp-uniform bases so that whole warps append together.
__global__ void __launch_bounds__(kThreads)
    k_roles_level(const BuildParams* __restrict__ params, const BVHNode32* __restrict__ lr,
                  const uint32_t* __restrict__ lrCount, const uint32_t* __restrict__ runStarts, uint32_t nTris,
                  int mergeMode, const uint32_t* __restrict__ frontIn, const uint32_t* __restrict__ countIn,
                  uint32_t* __restrict__ frontOut, uint32_t* countOut, uint8_t* __restrict__ role, uint32_t* errorWord)
{
  const uint32_t L = params->nLeaves;
  const uint32_t cap = L > 0 ? L - 1 : 0u;  // internal nodes, each a slot of one 4-wide node at most
  const uint32_t n = min(*countIn, cap);    // a count past the entries written is an error already reported
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warpBase = (blockIdx.x * kThreads + threadIdx.x) & ~31u;
  for (uint32_t b0 = warpBase; b0 < n; b0 += gridDim.x * kThreads)
  {
    const uint32_t f = b0 + lane;
    uint32_t next[4] = {0u, 0u, 0u, 0u};
    int cnt = 0;
    if (f < n)
    {
      uint32_t cand[4];
      const int nc = collapse_slots(lr, lrCount, L, kCollapseLargestFirst, frontIn[f], cand);
#pragma unroll
      for (int k = 0; k < 4; k++)
      {
        if (k >= nc) break;
        const uint32_t c = cand[k];
        if (c + 1u >= L) continue;  // a leaf slot
        const bool m = merges(lr, runStarts, L, nTris, mergeMode, c);
        role[c] = m ? 2 : 1;
        if (!m)
        {
#pragma unroll
          for (int j = 0; j < 4; j++)
            if (j == cnt) next[j] = c;
          cnt++;
        }
      }
    }
    warp_append(next, cnt, frontOut, countOut, cap, errorWord);
  }
}

// The root as the first level (L >= 2), every other level empty.
__global__ void k_roles_level_init(const BuildParams* __restrict__ params, uint32_t* __restrict__ front,
                                   uint32_t* __restrict__ counts, int levels, uint8_t* __restrict__ role)
{
  const uint32_t L = params->nLeaves;
  for (int k = threadIdx.x; k <= levels; k += blockDim.x) counts[k] = (k == 0 && L >= 2) ? 1u : 0u;
  if (threadIdx.x == 0 && L >= 2)
  {
    front[0] = 0;
    role[0] = 1;
  }
}

// A frontier left after the last level would mean a tree deeper than the
// depth bound: reported, never silently cut.
__global__ void k_roles_level_check(const uint32_t* __restrict__ counts, int levels, uint32_t* errorWord)
{
  if (counts[levels] != 0u) atomicOr(errorWord, kErrLayout);
}

// Depth bound of the largest-first levels: every 4-wide level descends at
// least one binary level, and a tree of distinct 30-bit codes is at most 31
// binary levels deep.
constexpr int kCollapseLevels = 34;

__global__ void __launch_bounds__(kThreads) k_roles(const BuildParams* __restrict__ params,
                                                    const BVHNode32* __restrict__ lr,
                                                    const uint32_t* __restrict__ runStarts, uint32_t nTris,
                                                    const uint8_t* __restrict__ depth, int mergeMode,
                                                    uint8_t* __restrict__ role)
{
  const uint32_t L = params->nLeaves;
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i + 1 < L; i += gridDim.x * kThreads)
    role[i] = node_role(lr, runStarts, L, nTris, depth[i], mergeMode, i);
}

// Exclusive scan of (role == 1) over the internal nodes: the 4-wide node index
// of each binary node that becomes one, in Karras order (the root gets 0); the
// prefix is written at every position.  n = L - 1 of params, or nGiven when
// params is null (the internal nodes of a whole batch, geometry after
// geometry).  One block per 4096 nodes, decoupled look-back as in the run
// compaction.
constexpr int      kScanItems  = 16;
constexpr uint32_t kScanTile   = kThreads * kScanItems;
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

__global__ void __launch_bounds__(kThreads) k_scan_roles(const BuildParams* __restrict__ params, uint32_t nGiven,
                                                         const uint8_t* __restrict__ role, uint32_t* __restrict__ index,
                                                         uint32_t* tileStatus, uint32_t* tileCounter, uint32_t* total,
                                                         uint32_t* errorWord)
{
  __shared__ uint32_t s_tile, s_prefix;
  __shared__ uint32_t s_warp[kThreads / 32 + 1];
  const uint32_t L = params ? params->nLeaves : 0u;
  const uint32_t n = params ? (L > 1 ? L - 1 : 0) : nGiven;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(tileCounter, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tile >= tiles) return;  // the grid is sized for the worst case
  const uint32_t base = tile * kScanTile + tid * kScanItems;
  uint32_t flags = 0, cnt = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
  {
    const uint32_t i = base + k;
    const bool f = i < n && role[i] == 1;
    flags |= (f ? 1u : 0u) << k;
    cnt += f ? 1u : 0u;
  }
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
    for (int w = 0; w < kThreads / 32; w++)
    {
      const uint32_t t = s_warp[w];
      s_warp[w] = run;
      run += t;
    }
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
    if (tile == tiles - 1) *total = excl + run;
  }
  __syncthreads();
  uint32_t pos = s_prefix + s_warp[warp] + incl - cnt;
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
  {
    const uint32_t i = base + k;
    if (i < n)
    {
      index[i] = pos;
      pos += (flags >> k) & 1u;
    }
  }
}

struct Slot
{
  float    lo[3], hi[3];
  uint32_t ref;  // node index, kLeafBit | first triangle, or kEmptyRef
};

__device__ __forceinline__ uint32_t h2_bits(__half lo, __half hi)
{
  return (uint32_t)__half_as_ushort(lo) | ((uint32_t)__half_as_ushort(hi) << 16);
}

// Smallest power-of-two exponent e with 255 * 2^e >= ext (e in [-126, 127]).
__device__ __forceinline__ int q8_exponent(float ext)
{
  if (!(ext > 0.0f)) return -126;
  int e;
  frexpf(ext / 255.0f, &e);  // ext/255 = m * 2^e, m in [0.5, 1)
  if (e < -126) e = -126;
  if (e > 127) e = 127;
  return e;
}

__device__ __forceinline__ float q8_scale(int e) { return __int_as_float((e + 127) << 23); }

// decoded bound = origin + q * 2^e (one product, exact for q < 256; one rounded add)
__device__ __forceinline__ float q8_decode(float origin, uint32_t q, float scale)
{
  return __fadd_rn(origin, __fmul_rn((float)q, scale));
}

__device__ __forceinline__ uint32_t q8_lo(float origin, float v, float scale)
{
  float qf = floorf(__fdiv_rn(__fsub_rn(v, origin), scale));
  int q = (int)fmaxf(0.0f, fminf(255.0f, qf));
  while (q > 0 && q8_decode(origin, (uint32_t)q, scale) > v) q--;
  return (uint32_t)q;
}

__device__ __forceinline__ uint32_t q8_hi(float origin, float v, float scale, bool& ok)
{
  float qf = ceilf(__fdiv_rn(__fsub_rn(v, origin), scale));
  int q = (int)fmaxf(0.0f, fminf(255.0f, qf));
  while (q < 255 && q8_decode(origin, (uint32_t)q, scale) < v) q++;
  ok = q8_decode(origin, (uint32_t)q, scale) >= v;
  return (uint32_t)q;
}

// One 4-wide node written in `format` (0 FP32, 1 FP16 rounded outward, 2
// 8-bit in a per-node frame) from its ns used slots.
__device__ __forceinline__ void write_node4(int format, void* __restrict__ nodes, uint32_t outIdx, Slot (&slot)[4],
                                            int ns, uint32_t* errorWord)
{
#pragma unroll
  for (int k = 0; k < 4; k++)
    if (k >= ns)
    {
      for (int c = 0; c < 3; c++) { slot[k].lo[c] = 0.0f; slot[k].hi[c] = 0.0f; }
      slot[k].ref = kEmptyRef;
    }
  if (format == 0)
  {
    Node4F32 o;
    o.lox = make_float4(slot[0].lo[0], slot[1].lo[0], slot[2].lo[0], slot[3].lo[0]);
    o.loy = make_float4(slot[0].lo[1], slot[1].lo[1], slot[2].lo[1], slot[3].lo[1]);
    o.loz = make_float4(slot[0].lo[2], slot[1].lo[2], slot[2].lo[2], slot[3].lo[2]);
    o.hix = make_float4(slot[0].hi[0], slot[1].hi[0], slot[2].hi[0], slot[3].hi[0]);
    o.hiy = make_float4(slot[0].hi[1], slot[1].hi[1], slot[2].hi[1], slot[3].hi[1]);
    o.hiz = make_float4(slot[0].hi[2], slot[1].hi[2], slot[2].hi[2], slot[3].hi[2]);
    o.ref = make_uint4(slot[0].ref, slot[1].ref, slot[2].ref, slot[3].ref);
    o.pad = make_uint4(0, 0, 0, 0);
    reinterpret_cast<Node4F32*>(nodes)[outIdx] = o;
  }
  else if (format == 1)
  {
    uint32_t w[12];
    for (int k = 0; k < 4; k++)
    {
      w[0 + k] = h2_bits(__float2half_rd(slot[k].lo[0]), __float2half_rd(slot[k].lo[1]));
      w[4 + k] = h2_bits(__float2half_rd(slot[k].lo[2]), __float2half_ru(slot[k].hi[0]));
      w[8 + k] = h2_bits(__float2half_ru(slot[k].hi[1]), __float2half_ru(slot[k].hi[2]));
    }
    Node4F16 o;
    o.a = make_uint4(w[0], w[1], w[2], w[3]);
    o.b = make_uint4(w[4], w[5], w[6], w[7]);
    o.c = make_uint4(w[8], w[9], w[10], w[11]);
    o.ref = make_uint4(slot[0].ref, slot[1].ref, slot[2].ref, slot[3].ref);
    reinterpret_cast<Node4F16*>(nodes)[outIdx] = o;
  }
  else
  {
    // frame: the union of the slots' boxes; per-axis power-of-two scale
    float org[3], scale[3];
    int ex[3];
    for (int c = 0; c < 3; c++)
    {
      float mn = slot[0].lo[c], mx = slot[0].hi[c];
      for (int k = 1; k < ns; k++)
      {
        mn = fminf(mn, slot[k].lo[c]);
        mx = fmaxf(mx, slot[k].hi[c]);
      }
      org[c] = mn;
      ex[c] = q8_exponent(__fsub_rn(mx, mn));
      // widen the scale until the frame's top is representable outward
      for (int guard = 0; guard < 4; guard++)
      {
        if (q8_decode(org[c], 255u, q8_scale(ex[c])) >= mx || ex[c] >= 127) break;
        ex[c]++;
      }
      scale[c] = q8_scale(ex[c]);
    }
    uint32_t qb[6] = {0, 0, 0, 0, 0, 0};  // lox, loy, loz, hix, hiy, hiz: 4 bytes each (one per slot)
    for (int k = 0; k < ns; k++)
      for (int c = 0; c < 3; c++)
      {
        bool ok = true;
        const uint32_t lo = q8_lo(org[c], slot[k].lo[c], scale[c]);
        const uint32_t hi = q8_hi(org[c], slot[k].hi[c], scale[c], ok);
        if (!ok) atomicOr(errorWord, kErrLayout);
        qb[c] |= lo << (8 * k);
        qb[3 + c] |= hi << (8 * k);
      }
    Node4Q8 o;
    o.frame = make_float4(org[0], org[1], org[2],
                          __uint_as_float((uint32_t)(ex[0] + 128) | ((uint32_t)(ex[1] + 128) << 8) |
                                          ((uint32_t)(ex[2] + 128) << 16)));
    o.q0 = make_uint4(qb[0], qb[1], qb[2], qb[3]);
    o.q1 = make_uint4(qb[4], qb[5], 0u, 0u);
    o.ref = make_uint4(slot[0].ref, slot[1].ref, slot[2].ref, slot[3].ref);
    reinterpret_cast<Node4Q8*>(nodes)[outIdx] = o;
  }
}

// The slots of the 4-wide node that binary node i (role 1) of one tree becomes:
// its grandchildren, or a child itself when that child is a leaf.  A slot is a
// leaf (kLeafBit | first triangle), a merged leaf (role 2: its runs joined, the
// 4-wide end flag cleared at the ends of the runs before the last), or the
// 4-wide node indexOf(child) of another role-1 node.  With one leaf (L == 1)
// the node holds that leaf alone.  Returns the number of used slots.
template <typename IndexOf>
__device__ __forceinline__ int node4_slots(const BVHNode32* __restrict__ lr, const uint32_t* __restrict__ lrCount,
                                           const uint32_t* __restrict__ runStarts, uint32_t L, uint32_t nTris,
                                           int collapse, const uint8_t* __restrict__ role, IndexOf indexOf, uint32_t i,
                                           TriRec* __restrict__ tris, Slot (&slot)[4])
{
  if (L == 1u)
  {
    const BVHNode32 n = lr[0];
    for (int c = 0; c < 3; c++) { slot[0].lo[c] = n.boxMin[c]; slot[0].hi[c] = n.boxMax[c]; }
    slot[0].ref = kLeafBit | runStarts[0];
    return 1;
  }
  uint32_t cand[4];
  const int nc = collapse_slots(lr, lrCount, L, collapse, i, cand);
#pragma unroll
  for (int k = 0; k < 4; k++)
  {
    if (k >= nc) break;
    const uint32_t s = cand[k];
    const BVHNode32 n = lr[s];
    for (int c = 0; c < 3; c++) { slot[k].lo[c] = n.boxMin[c]; slot[k].hi[c] = n.boxMax[c]; }
    if (s + 1u >= L)
      slot[k].ref = kLeafBit | runStarts[s - (L - 1)];
    else if (role[s] == 2)
    {
      uint32_t st, en;
      node_range(lr, runStarts, L, nTris, s, st, en);
      slot[k].ref = kLeafBit | st;
      uint32_t a = s, b = s;
      while (a + 1u < L) a = lr[a].leftOffset;
      while (b + 1u < L) b = lr[b].escapeIndex;
      for (uint32_t leaf = a - (L - 1); leaf < b - (L - 1); leaf++)
      {
        const uint32_t runEnd = runStarts[leaf + 1];
        if (runEnd > st && runEnd < en)
        {
          const uint32_t w = __float_as_uint(tris[runEnd - 1].a.w);
          tris[runEnd - 1].a.w = __uint_as_float(w & ~2u);
        }
      }
    }
    else
      slot[k].ref = indexOf(s);
  }
  return nc;
}

__global__ void __launch_bounds__(kThreads) k_emit4(const BuildParams* __restrict__ params,
                                                    const BVHNode32* __restrict__ lr,
                                                    const uint32_t* __restrict__ lrCount,
                                                    const uint32_t* __restrict__ runStarts, uint32_t nTris,
                                                    int collapse, const uint8_t* __restrict__ role,
                                                    const uint32_t* __restrict__ index, int format,
                                                    void* __restrict__ nodes, uint32_t maxNodes,
                                                    TriRec* __restrict__ tris, uint32_t* errorWord)
{
  const uint32_t L = params->nLeaves;
  const uint32_t first = blockIdx.x * kThreads + threadIdx.x;
  const uint32_t count = (L == 1u) ? 1u : L - 1u;
  for (uint32_t i = first; i < count; i += gridDim.x * kThreads)
  {
    uint32_t outIdx = 0;
    if (L != 1u)
    {
      if (role[i] != 1) continue;
      outIdx = index[i];
      if (outIdx >= maxNodes)  // only after a failed numbering (reported through the error word)
      {
        atomicOr(errorWord, kErrLayout);
        continue;
      }
    }
    Slot slot[4];
    const int ns = node4_slots(lr, lrCount, runStarts, L, nTris, collapse, role, [&](uint32_t c) { return index[c]; },
                               i, tris, slot);
    write_node4(format, nodes, outIdx, slot, ns, errorWord);
  }
}

// ---------------------------------------------------------------- batches
// The same collapse for the geometries of a segmented build at once: internal
// node j of the batch is node j - intOffsets[s] of geometry s; each geometry's
// 4-wide nodes are numbered from 0 (its root) and stored at node4Off[s].
struct SegTree
{
  const BVHNode32* lr;
  const uint32_t*  lrCount;
  const uint32_t*  runStarts;
  const uint32_t*  parent;
  TriRec*          tris;
  uint32_t         L, nTris, intBase, seg;
};

__device__ __forceinline__ SegTree seg_tree(const Bvh4Batch& b, uint32_t seg)
{
  SegTree t;
  t.seg = seg;
  t.lr = b.lr + b.nodeOffsets[seg];
  t.lrCount = b.lrCount + b.nodeOffsets[seg];
  t.parent = b.parent + b.nodeOffsets[seg];
  t.runStarts = b.runStarts + b.leafOffsets[seg];
  t.tris = b.tris + b.triOffsets[seg];
  t.L = b.leafOffsets[seg + 1] - b.leafOffsets[seg];
  t.nTris = b.triOffsets[seg + 1] - b.triOffsets[seg];
  t.intBase = b.intOffsets[seg];
  return t;
}

__global__ void __launch_bounds__(kThreads) k_seg4_depth_roles(Bvh4Batch b, uint32_t nInt, uint8_t* __restrict__ role)
{
  for (uint32_t j = blockIdx.x * kThreads + threadIdx.x; j < nInt; j += gridDim.x * kThreads)
  {
    const SegTree t = seg_tree(b, bc::find_segment(b.intOffsets, b.G, j));
    const uint32_t i = j - t.intBase;
    role[j] = node_role(t.lr, t.runStarts, t.L, t.nTris, node_depth(t.parent, t.L, i), b.mergeMode, i);
  }
}

// Largest-first roles of a batch: the geometries' roots as the first level
// (batch-wide internal node indices), then one launch per level.
__global__ void __launch_bounds__(kThreads) k_seg4_roles_init(Bvh4Batch b, uint32_t* __restrict__ front,
                                                              uint32_t* counts, int levels, uint8_t* __restrict__ role)
{
  const uint32_t tid = blockIdx.x * kThreads + threadIdx.x;
  if (tid == 0)
    for (int k = 1; k <= levels; k++) counts[k] = 0u;
  for (uint32_t seg = tid; seg < b.G; seg += gridDim.x * kThreads)
    if (b.leafOffsets[seg + 1] - b.leafOffsets[seg] >= 2u)
    {
      const uint32_t j = b.intOffsets[seg];
      role[j] = 1;
      front[atomicAdd(counts, 1u)] = j;
    }
}

__global__ void __launch_bounds__(kThreads)
    k_seg4_roles_level(Bvh4Batch b, uint32_t nInt, const uint32_t* __restrict__ frontIn,
                       const uint32_t* __restrict__ countIn, uint32_t* __restrict__ frontOut, uint32_t* countOut,
                       uint8_t* __restrict__ role, uint32_t* errorWord)
{
  const uint32_t n = min(*countIn, nInt);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warpBase = (blockIdx.x * kThreads + threadIdx.x) & ~31u;
  for (uint32_t b0 = warpBase; b0 < n; b0 += gridDim.x * kThreads)
  {
    const uint32_t f = b0 + lane;
    uint32_t next[4] = {0u, 0u, 0u, 0u};
    int cnt = 0;
    if (f < n)
    {
      const uint32_t j = frontIn[f];
      const SegTree t = seg_tree(b, bc::find_segment(b.intOffsets, b.G, j));
      uint32_t cand[4];
      const int nc = collapse_slots(t.lr, t.lrCount, t.L, kCollapseLargestFirst, j - t.intBase, cand);
#pragma unroll
      for (int k = 0; k < 4; k++)
      {
        if (k >= nc) break;
        const uint32_t c = cand[k];
        if (c + 1u >= t.L) continue;
        const bool m = merges(t.lr, t.runStarts, t.L, t.nTris, b.mergeMode, c);
        role[t.intBase + c] = m ? 2 : 1;
        if (!m)
        {
#pragma unroll
          for (int q = 0; q < 4; q++)
            if (q == cnt) next[q] = t.intBase + c;
          cnt++;
        }
      }
    }
    warp_append(next, cnt, frontOut, countOut, nInt, errorWord);
  }
}

// Per geometry: its 4-wide node count (role-1 nodes; 1 for a single leaf; 0
// without triangles), its first node's batch-wide rank, and the exclusive sum
// of the counts (node4Off), in one block.  out: rootRank[G], count4[G],
// node4Off[G + 1].
__global__ void __launch_bounds__(1024) k_seg4_counts(Bvh4Batch b, uint32_t nInt, const uint32_t* __restrict__ rank,
                                                      const uint32_t* __restrict__ rankTotal, uint32_t* rootRank,
                                                      uint32_t* count4, uint32_t* node4Off)
{
  __shared__ uint32_t s_part[1024];
  __shared__ uint32_t s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < b.G; base += blockDim.x)
  {
    const uint32_t s = base + threadIdx.x;
    uint32_t c = 0;
    if (s < b.G)
    {
      const uint32_t L = b.leafOffsets[s + 1] - b.leafOffsets[s];
      const uint32_t j0 = b.intOffsets[s], j1 = b.intOffsets[s + 1];
      const uint32_t r0 = j0 < nInt ? rank[j0] : *rankTotal;
      const uint32_t r1 = j1 < nInt ? rank[j1] : *rankTotal;
      c = L > 1 ? r1 - r0 : (L == 1 ? 1u : 0u);
      rootRank[s] = r0;
      count4[s] = c;
    }
    s_part[threadIdx.x] = c;
    __syncthreads();
    for (uint32_t o = 1; o < blockDim.x; o <<= 1)
    {
      const uint32_t y = threadIdx.x >= o ? s_part[threadIdx.x - o] : 0u;
      __syncthreads();
      s_part[threadIdx.x] += y;
      __syncthreads();
    }
    if (s < b.G) node4Off[s] = s_carry + s_part[threadIdx.x] - c;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry += s_part[blockDim.x - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) node4Off[b.G] = s_carry;
}

// Threads j < nInt emit the role-1 internal nodes; threads nInt + s emit the
// lone-leaf node of geometry s when it has exactly one leaf.
__global__ void __launch_bounds__(kThreads) k_seg4_emit(Bvh4Batch b, uint32_t nInt, const uint8_t* __restrict__ role,
                                                        const uint32_t* __restrict__ rank,
                                                        const uint32_t* __restrict__ rootRank,
                                                        const uint32_t* __restrict__ node4Off, int format,
                                                        void* __restrict__ nodes, uint32_t* errorWord)
{
  for (uint32_t j = blockIdx.x * kThreads + threadIdx.x; j < nInt + b.G; j += gridDim.x * kThreads)
  {
    uint32_t seg, i;
    if (j < nInt)
    {
      if (role[j] != 1) continue;
      seg = bc::find_segment(b.intOffsets, b.G, j);
      i = j - b.intOffsets[seg];
    }
    else
    {
      seg = j - nInt;
      if (b.leafOffsets[seg + 1] - b.leafOffsets[seg] != 1u) continue;
      i = 0;
    }
    const SegTree t = seg_tree(b, seg);
    const uint32_t r0 = rootRank[seg];
    const uint32_t local = t.L == 1u ? 0u : rank[j] - r0;
    const uint32_t outIdx = node4Off[seg] + local;
    if (outIdx >= node4Off[seg + 1])
    {
      atomicOr(errorWord, kErrLayout);
      continue;
    }
    Slot slot[4];
    const uint8_t* roleSeg = role + t.intBase;
    const uint32_t* rankSeg = rank + t.intBase;
    const int ns = node4_slots(t.lr, t.lrCount, t.runStarts, t.L, t.nTris, b.collapse, roleSeg,
                               [&](uint32_t c) { return rankSeg[c] - r0; }, i, t.tris, slot);
    write_node4(format, nodes, outIdx, slot, ns, errorWord);
  }
}

inline uint32_t grid_for(uint64_t n, int numSMs)
{
  uint64_t g = (n + kThreads - 1) / kThreads;
  const uint64_t cap = (uint64_t)numSMs * 8;
  if (g > cap) g = cap;
  return g == 0 ? 1u : (uint32_t)g;
}

// Blocks for level `lvl` of the largest-first roles: the level holds at most
// roots * 4^lvl entries (and never more than the internal nodes); the loop
// strides over larger levels, so two blocks per SM suffice.
inline uint32_t level_grid(int lvl, uint64_t roots, uint64_t nInternal, int numSMs)
{
  uint64_t most = roots;
  for (int k = 0; k < lvl && most < nInternal; k++) most *= 4;
  if (most > nInternal) most = nInternal;
  uint64_t g = (most + kThreads - 1) / kThreads;
  const uint64_t cap = (uint64_t)numSMs * 2;
  if (g > cap) g = cap;
  return g == 0 ? 1u : (uint32_t)g;
}

}  // namespace

// Scratch: total (256 B), depth and role (N B each), index (4N B; also the
// first frontier of the largest-first roles), scan tile status, the second
// frontier (4N B) and the level counts.
size_t bvh4_scratch_bytes(uint32_t nTris)
{
  const size_t n = nTris ? nTris : 1;
  const size_t tiles = (n + kScanTile - 1) / kScanTile;
  return 256 + ((2 * n + 255) / 256) * 256 + ((4 * n + 255) / 256) * 256 + ((4 * (tiles + 8) + 255) / 256) * 256 +
         ((4 * n + 255) / 256) * 256 + 4 * (kCollapseLevels + 1);
}

namespace
{
struct SingleScratch
{
  uint32_t *total, *index, *tiles, *front2, *levelCounts;
  uint8_t *depth, *role;
};
SingleScratch single_scratch(void* scratch, uint32_t N)
{
  const size_t n = N ? N : 1;
  const size_t tiles = (n + kScanTile - 1) / kScanTile;
  char* p = (char*)scratch;
  SingleScratch q;
  q.total = (uint32_t*)p;
  q.depth = (uint8_t*)(p + 256);
  q.role = q.depth + N;
  q.index = (uint32_t*)(p + 256 + ((2 * n + 255) / 256) * 256);
  q.tiles = (uint32_t*)((char*)q.index + ((4 * n + 255) / 256) * 256);
  q.front2 = (uint32_t*)((char*)q.tiles + ((4 * (tiles + 8) + 255) / 256) * 256);
  q.levelCounts = (uint32_t*)((char*)q.front2 + ((4 * n + 255) / 256) * 256);
  return q;
}
}  // namespace

cudaError_t bvh4_plan(const Bvh4Buffers& b, int numSMs, cudaStream_t s)
{
  const uint32_t N = b.nTris;
  const SingleScratch q = single_scratch(b.scratch, N);
  const size_t nTiles = ((size_t)N + kScanTile - 1) / kScanTile;
  cudaError_t e = cudaMemsetAsync(q.total, 0, 4, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(q.tiles, 0, 4 * (nTiles + 8), s);
  if (e != cudaSuccess) return e;
  const uint32_t g = grid_for(N, numSMs);
  if (b.collapse == kCollapseLargestFirst)
  {
    e = cudaMemsetAsync(q.role, 0, N ? N : 1, s);
    if (e != cudaSuccess) return e;
    k_roles_level_init<<<1, 64, 0, s>>>(b.params, q.index, q.levelCounts, kCollapseLevels, q.role);
    for (int lvl = 0; lvl < kCollapseLevels; lvl++)
    {
      uint32_t* in = (lvl & 1) ? q.front2 : q.index;
      uint32_t* out = (lvl & 1) ? q.index : q.front2;
      k_roles_level<<<level_grid(lvl, 1, N, numSMs), kThreads, 0, s>>>(
          b.params, b.lr, b.lrCount, b.runStarts, N, b.mergeMode, in, q.levelCounts + lvl, out,
          q.levelCounts + lvl + 1, q.role, &b.params->error);
    }
    k_roles_level_check<<<1, 1, 0, s>>>(q.levelCounts, kCollapseLevels, &b.params->error);
  }
  else
  {
    k_depth<<<g, kThreads, 0, s>>>(b.params, b.parent, q.depth);
    k_roles<<<g, kThreads, 0, s>>>(b.params, b.lr, b.runStarts, N, q.depth, b.mergeMode, q.role);
  }
  k_scan_roles<<<(uint32_t)(nTiles ? nTiles : 1), kThreads, 0, s>>>(b.params, 0u, q.role, q.index, q.tiles + 4,
                                                                      q.tiles, q.total, &b.params->error);
  return cudaMemcpyAsync(b.hostNodeCount, q.total, 4, cudaMemcpyDeviceToHost, s);
}

cudaError_t bvh4_emit(const Bvh4Buffers& b, int format, void* nodes, uint32_t maxNodes, int numSMs, cudaStream_t s)
{
  const uint32_t N = b.nTris;
  const SingleScratch q = single_scratch(b.scratch, N);
  k_emit4<<<grid_for(N, numSMs), kThreads, 0, s>>>(b.params, b.lr, b.lrCount, b.runStarts, N, b.collapse, q.role,
                                                   q.index, format, nodes, maxNodes, b.tris, &b.params->error);
  return cudaGetLastError();
}

// Batch scratch: total (256 B), role (nInt B), rank (4 nInt B; also the
// first frontier of the largest-first roles), per-geometry rootRank, count4,
// node4Off (4 (3G + 1) B), scan tile status, the second frontier (4 nInt B)
// and the level counts.
size_t bvh4_batch_scratch_bytes(uint32_t nInt, uint32_t G)
{
  const size_t n = nInt ? nInt : 1;
  const size_t tiles = (n + kScanTile - 1) / kScanTile;
  return 256 + ((n + 255) / 256) * 256 + ((4 * n + 255) / 256) * 256 + ((4 * (3 * (size_t)G + 1) + 255) / 256) * 256 +
         ((4 * (tiles + 8) + 255) / 256) * 256 + ((4 * n + 255) / 256) * 256 + 4 * (kCollapseLevels + 1);
}

namespace
{
struct BatchScratch
{
  uint32_t *total, *rank, *rootRank, *count4, *node4Off, *tiles, *front2, *levelCounts;
  uint8_t* role;
};
BatchScratch batch_scratch(void* scratch, uint32_t nInt, uint32_t G)
{
  const size_t n = nInt ? nInt : 1;
  const size_t tiles = (n + kScanTile - 1) / kScanTile;
  char* p = (char*)scratch;
  BatchScratch q;
  q.total = (uint32_t*)p;
  q.role = (uint8_t*)(p + 256);
  q.rank = (uint32_t*)(p + 256 + ((n + 255) / 256) * 256);
  q.rootRank = (uint32_t*)((char*)q.rank + ((4 * n + 255) / 256) * 256);
  q.count4 = q.rootRank + G;
  q.node4Off = q.count4 + G;
  q.tiles = (uint32_t*)((char*)q.rootRank + ((4 * (3 * (size_t)G + 1) + 255) / 256) * 256);
  q.front2 = (uint32_t*)((char*)q.tiles + ((4 * (tiles + 8) + 255) / 256) * 256);
  q.levelCounts = (uint32_t*)((char*)q.front2 + ((4 * n + 255) / 256) * 256);
  return q;
}
}  // namespace

cudaError_t bvh4_plan_batch(const Bvh4Batch& b, uint32_t nInt, void* scratch, uint32_t* hostCount4,
                            uint32_t* hostNode4Off, uint32_t* errorWord, int numSMs, cudaStream_t s)
{
  const BatchScratch q = batch_scratch(scratch, nInt, b.G);
  const size_t nTiles = ((size_t)(nInt ? nInt : 1) + kScanTile - 1) / kScanTile;
  cudaError_t e = cudaMemsetAsync(q.total, 0, 4, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(q.tiles, 0, 4 * (nTiles + 8), s);
  if (e != cudaSuccess) return e;
  if (nInt)
  {
    if (b.collapse == kCollapseLargestFirst)
    {
      e = cudaMemsetAsync(q.role, 0, nInt, s);
      if (e != cudaSuccess) return e;
      e = cudaMemsetAsync(q.levelCounts, 0, 4, s);
      if (e != cudaSuccess) return e;
      k_seg4_roles_init<<<grid_for(b.G, numSMs), kThreads, 0, s>>>(b, q.rank, q.levelCounts, kCollapseLevels, q.role);
      for (int lvl = 0; lvl < kCollapseLevels; lvl++)
      {
        uint32_t* in = (lvl & 1) ? q.front2 : q.rank;
        uint32_t* out = (lvl & 1) ? q.rank : q.front2;
        k_seg4_roles_level<<<level_grid(lvl, b.G, nInt, numSMs), kThreads, 0, s>>>(
            b, nInt, in, q.levelCounts + lvl, out, q.levelCounts + lvl + 1, q.role, errorWord);
      }
      k_roles_level_check<<<1, 1, 0, s>>>(q.levelCounts, kCollapseLevels, errorWord);
    }
    else
      k_seg4_depth_roles<<<grid_for(nInt, numSMs), kThreads, 0, s>>>(b, nInt, q.role);
    k_scan_roles<<<(uint32_t)nTiles, kThreads, 0, s>>>(nullptr, nInt, q.role, q.rank, q.tiles + 4, q.tiles, q.total,
                                                       errorWord);
  }
  k_seg4_counts<<<1, 1024, 0, s>>>(b, nInt, q.rank, q.total, q.rootRank, q.count4, q.node4Off);
  e = cudaMemcpyAsync(hostCount4, q.count4, 4 * (size_t)b.G, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(hostNode4Off, q.node4Off, 4 * ((size_t)b.G + 1), cudaMemcpyDeviceToHost, s);
}

cudaError_t bvh4_emit_batch(const Bvh4Batch& b, uint32_t nInt, void* scratch, int format, void* nodes,
                            uint32_t* errorWord, int numSMs, cudaStream_t s)
{
  const BatchScratch q = batch_scratch(scratch, nInt, b.G);
  k_seg4_emit<<<grid_for((uint64_t)nInt + b.G, numSMs), kThreads, 0, s>>>(b, nInt, q.role, q.rank, q.rootRank,
                                                                           q.node4Off, format, nodes, errorWord);
  return cudaGetLastError();
}

}  // namespace hrt
