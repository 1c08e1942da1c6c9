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
// Quantised boxes only ever contain the FP32 box they stand for, so a
// traversal of the quantised tree visits every node the FP32 tree would and
// can only add visits; the triangle test is unchanged.
#include <cuda_fp16.h>

#include "hrt_kernels.cuh"

namespace hrt
{
namespace
{

constexpr int kThreads = 256;

// Depth of every internal node: walk up the parent chain (depth <= 30).
__global__ void __launch_bounds__(kThreads) k_depth(const BuildParams* __restrict__ params,
                                                    const uint32_t* __restrict__ parent, uint8_t* __restrict__ depth)
{
  const uint32_t L = params->nLeaves;
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i + 1 < L; i += gridDim.x * kThreads)
  {
    uint32_t d = 0, n = i;
    while (n != 0 && d < 255)
    {
      const uint32_t p = parent[n];
      if (p + 1u >= L) break;  // only the root lacks an internal parent
      n = p;
      d++;
    }
    depth[i] = (uint8_t)d;
  }
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

// Role of each internal node: 1 = 4-wide node, 2 = merged leaf, 0 = absorbed.
// mergeMode 0: merge when both children are leaves (the reference's rule);
// mergeMode M > 0: merge when the subtree holds at most M triangles.
__global__ void __launch_bounds__(kThreads) k_roles(const BuildParams* __restrict__ params,
                                                    const BVHNode32* __restrict__ lr,
                                                    const uint32_t* __restrict__ runStarts, uint32_t nTris,
                                                    const uint8_t* __restrict__ depth, int mergeMode,
                                                    uint8_t* __restrict__ role)
{
  const uint32_t L = params->nLeaves;
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i + 1 < L; i += gridDim.x * kThreads)
  {
    uint8_t r = 0;
    if ((depth[i] & 1u) == 0u)
    {
      bool merge;
      if (mergeMode == 0)
        merge = lr[i].leftOffset + 1u >= L && lr[i].escapeIndex + 1u >= L;
      else
      {
        uint32_t st, en;
        node_range(lr, runStarts, L, nTris, i, st, en);
        merge = en - st <= (uint32_t)mergeMode;
      }
      r = (i != 0 && merge) ? 2 : 1;
    }
    role[i] = r;
  }
}

// Exclusive scan of (role == 1) over the internal nodes: the 4-wide node index
// of each binary node that becomes one, in Karras order (the root gets 0).
// One block per 4096 nodes, decoupled look-back as in the run compaction.
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

__global__ void __launch_bounds__(kThreads) k_scan_roles(const BuildParams* __restrict__ params,
                                                         const uint8_t* __restrict__ role, uint32_t* __restrict__ index,
                                                         uint32_t* tileStatus, uint32_t* tileCounter, uint32_t* total,
                                                         uint32_t* errorWord)
{
  __shared__ uint32_t s_tile, s_prefix;
  __shared__ uint32_t s_warp[kThreads / 32 + 1];
  const uint32_t L = params->nLeaves;
  const uint32_t n = L > 1 ? L - 1 : 0;
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
    if (i < n) index[i] = (flags & (1u << k)) ? pos++ : 0xFFFFFFFFu;
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

__global__ void __launch_bounds__(kThreads) k_emit4(const BuildParams* __restrict__ params,
                                                    const BVHNode32* __restrict__ lr,
                                                    const uint32_t* __restrict__ runStarts, uint32_t nTris,
                                                    const uint8_t* __restrict__ role, const uint32_t* __restrict__ index,
                                                    int format, void* __restrict__ nodes, uint32_t maxNodes,
                                                    TriRec* __restrict__ tris, uint32_t* errorWord)
{
  const uint32_t L = params->nLeaves;
  const uint32_t first = blockIdx.x * kThreads + threadIdx.x;
  const uint32_t count = (L == 1u) ? 1u : L - 1u;
  for (uint32_t i = first; i < count; i += gridDim.x * kThreads)
  {
    Slot slot[4];
    int ns = 0;
    uint32_t outIdx;
    if (L == 1u)
    {
      outIdx = 0;
      const BVHNode32 n = lr[0];
      for (int c = 0; c < 3; c++) { slot[0].lo[c] = n.boxMin[c]; slot[0].hi[c] = n.boxMax[c]; }
      slot[0].ref = kLeafBit | runStarts[0];
      ns = 1;
    }
    else
    {
      if (role[i] != 1) continue;
      outIdx = index[i];
      if (outIdx >= maxNodes)  // only after a failed numbering (reported through the error word)
      {
        atomicOr(errorWord, kErrLayout);
        continue;
      }
      const uint32_t kids[2] = {lr[i].leftOffset, lr[i].escapeIndex};
      uint32_t cand[4];
      int nc = 0;
      for (int k = 0; k < 2; k++)
      {
        const uint32_t c = kids[k];
        if (c + 1u >= L)
          cand[nc++] = c;
        else
        {
          cand[nc++] = lr[c].leftOffset;
          cand[nc++] = lr[c].escapeIndex;
        }
      }
      for (int k = 0; k < nc; k++)
      {
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
          // the merged leaf ends at the end of its last run: clear the 4-wide
          // end flag (bit 1) at the ends of the runs before it
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
          slot[k].ref = index[s];
      }
      ns = nc;
    }
    for (int k = ns; k < 4; k++)
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
}

inline uint32_t grid_for(uint64_t n, int numSMs)
{
  uint64_t g = (n + kThreads - 1) / kThreads;
  const uint64_t cap = (uint64_t)numSMs * 8;
  if (g > cap) g = cap;
  return g == 0 ? 1u : (uint32_t)g;
}

}  // namespace

size_t bvh4_scratch_bytes(uint32_t nTris)
{
  const size_t n = nTris ? nTris : 1;
  const size_t tiles = (n + kScanTile - 1) / kScanTile;
  return 256 + ((2 * n + 255) / 256) * 256 + ((4 * n + 255) / 256) * 256 + 4 * (tiles + 8);
}

cudaError_t bvh4_plan(const Bvh4Buffers& b, int numSMs, cudaStream_t s)
{
  const uint32_t N = b.nTris;
  char* p = (char*)b.scratch;
  uint32_t* total = (uint32_t*)p;
  uint8_t* depth = (uint8_t*)(p + 256);
  uint8_t* role = depth + N;
  uint32_t* index = (uint32_t*)(p + 256 + ((2 * (size_t)N + 255) / 256) * 256);
  uint32_t* tiles = index + ((4 * (size_t)N + 255) / 256) * 64;
  const size_t nTiles = ((size_t)N + kScanTile - 1) / kScanTile;
  cudaError_t e = cudaMemsetAsync(total, 0, 4, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(tiles, 0, 4 * (nTiles + 8), s);
  if (e != cudaSuccess) return e;
  const uint32_t g = grid_for(N, numSMs);
  k_depth<<<g, kThreads, 0, s>>>(b.params, b.parent, depth);
  k_roles<<<g, kThreads, 0, s>>>(b.params, b.lr, b.runStarts, N, depth, b.mergeMode, role);
  k_scan_roles<<<(uint32_t)(nTiles ? nTiles : 1), kThreads, 0, s>>>(b.params, role, index, tiles + 4, tiles, total,
                                                                      &b.params->error);
  return cudaMemcpyAsync(b.hostNodeCount, total, 4, cudaMemcpyDeviceToHost, s);
}

cudaError_t bvh4_emit(const Bvh4Buffers& b, int format, void* nodes, uint32_t maxNodes, int numSMs, cudaStream_t s)
{
  const uint32_t N = b.nTris;
  char* p = (char*)b.scratch;
  uint8_t* depth = (uint8_t*)(p + 256);
  uint8_t* role = depth + N;
  uint32_t* index = (uint32_t*)(p + 256 + ((2 * (size_t)N + 255) / 256) * 256);
  k_emit4<<<grid_for(N, numSMs), kThreads, 0, s>>>(b.params, b.lr, b.runStarts, N, role, index, format, nodes,
                                                   maxNodes, b.tris, &b.params->error);
  return cudaGetLastError();
}

}  // namespace hrt
