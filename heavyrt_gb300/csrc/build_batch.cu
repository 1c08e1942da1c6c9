// Segmented LBVH build: many independent geometries built by one launch per
// stage over their concatenated triangles.
//
// Every geometry gets exactly the arrays its single build would produce (same
// scene box, Morton codes, stable order, runs, Karras tree, refit boxes and
// traversal records) at its own offsets:
//   triangles  [triOffsets[s], triOffsets[s+1])            keys, vals, TriRec, sorted index buffer
//   runs       [leafOffsets[s], leafOffsets[s+1])          compressed codes, run starts
//   LR nodes   [nodeOffsets[s], nodeOffsets[s] + 2L-1)     Karras + refit tree, local numbering
//   records    [recOffsets[s], recOffsets[s] + max(L-1,1)) child-pair records, local references
// The per-geometry box uses the geometry's own vertices and the centroid rule
// uses the geometry's own triangle count (core/builders/lbvh.cpp:279); the
// sort is the stable segmented radix sort; a run never crosses a segment.
#include "build_common.cuh"
#include "hrt_kernels.cuh"

namespace hrt
{
namespace
{

constexpr int kThreads = 256;
using bc::find_segment;

// Scene box and Morton scale of each geometry, in two passes: every geometry's
// vertices in chunks of kBoxChunk, one block per chunk (geometry s owns chunks
// [chunkOffsets[s], chunkOffsets[s + 1])), then the chunks of each geometry
// combined in order.  Min / max are exact, so the box is the reference's
// (core/builders/lbvh.cpp:228-239; init +-1e10, :53).
constexpr uint32_t kBoxChunk = kBatchBoxChunk;

__global__ void __launch_bounds__(kThreads) k_seg_box_partial(const float4* __restrict__ v,
                                                              const uint32_t* __restrict__ vertOffsets,
                                                              const uint32_t* __restrict__ chunkOffsets, uint32_t G,
                                                              float4* __restrict__ partial)
{
  const uint32_t k = blockIdx.x;
  const uint32_t s = find_segment(chunkOffsets, G, k);
  const uint32_t c = k - chunkOffsets[s];
  const uint32_t b = vertOffsets[s] + c * kBoxChunk;
  const uint32_t e = min(b + kBoxChunk, vertOffsets[s + 1]);
  float mn[4] = {1e10f, 1e10f, 1e10f, 1e10f}, mx[4] = {-1e10f, -1e10f, -1e10f, -1e10f};
  for (uint32_t i = b + threadIdx.x; i < e; i += kThreads)
  {
    const float4 p = v[i];
    mn[0] = lm_min(mn[0], p.x); mn[1] = lm_min(mn[1], p.y); mn[2] = lm_min(mn[2], p.z); mn[3] = lm_min(mn[3], p.w);
    mx[0] = lm_max(mx[0], p.x); mx[1] = lm_max(mx[1], p.y); mx[2] = lm_max(mx[2], p.z); mx[3] = lm_max(mx[3], p.w);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < 4; q++)
    {
      mn[q] = lm_min(mn[q], __shfl_down_sync(0xFFFFFFFFu, mn[q], o));
      mx[q] = lm_max(mx[q], __shfl_down_sync(0xFFFFFFFFu, mx[q], o));
    }
  __shared__ float smn[kThreads / 32][4], smx[kThreads / 32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int q = 0; q < 4; q++) { smn[warp][q] = mn[q]; smx[warp][q] = mx[q]; }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    for (int w = 1; w < kThreads / 32; w++)
      for (int q = 0; q < 4; q++) { mn[q] = lm_min(mn[q], smn[w][q]); mx[q] = lm_max(mx[q], smx[w][q]); }
    partial[2 * k] = make_float4(mn[0], mn[1], mn[2], mn[3]);
    partial[2 * k + 1] = make_float4(mx[0], mx[1], mx[2], mx[3]);
  }
}

__global__ void __launch_bounds__(kThreads) k_seg_box_final(const uint32_t* __restrict__ chunkOffsets, uint32_t G,
                                                            const float4* __restrict__ partial, BuildParams* params,
                                                            int cubic)
{
  for (uint32_t s = blockIdx.x * kThreads + threadIdx.x; s < G; s += gridDim.x * kThreads)
  {
    float mn[4] = {1e10f, 1e10f, 1e10f, 1e10f}, mx[4] = {-1e10f, -1e10f, -1e10f, -1e10f};
    for (uint32_t k = chunkOffsets[s]; k < chunkOffsets[s + 1]; k++)
    {
      const float4 a = partial[2 * k], b = partial[2 * k + 1];
      mn[0] = lm_min(mn[0], a.x); mn[1] = lm_min(mn[1], a.y); mn[2] = lm_min(mn[2], a.z); mn[3] = lm_min(mn[3], a.w);
      mx[0] = lm_max(mx[0], b.x); mx[1] = lm_max(mx[1], b.y); mx[2] = lm_max(mx[2], b.z); mx[3] = lm_max(mx[3], b.w);
    }
    bc::zindex_scale(mn, mx, &params[s], cubic);
    params[s].nLeaves = 0;
    params[s].error = 0;
  }
}

__global__ void __launch_bounds__(kThreads) k_seg_morton(const float4* __restrict__ v, const uint32_t* __restrict__ idx,
                                                         const uint32_t* __restrict__ vertOffsets,
                                                         const uint32_t* __restrict__ triOffsets, uint32_t G,
                                                         uint32_t N, const BuildParams* __restrict__ params,
                                                         uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                         uint32_t* errorWord)
{
  const uint32_t t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= N) return;
  const uint32_t s = find_segment(triOffsets, G, t);
  const uint32_t nT = triOffsets[s + 1] - triOffsets[s];
  const uint32_t vb = vertOffsets[s], nV = vertOffsets[s + 1] - vb;
  uint32_t ia = idx[3 * (size_t)t + 0], ib = idx[3 * (size_t)t + 1], ic = idx[3 * (size_t)t + 2];
  if (ia >= nV || ib >= nV || ic >= nV)
  {
    atomicOr(errorWord, kErrIndexRange);
    ia = ib = ic = 0;
  }
  keys[t] = bc::morton_code(v[vb + ia], v[vb + ib], v[vb + ic], nT, params[s].bmin, params[s].scale);
  vals[t] = t;
}

__global__ void __launch_bounds__(kThreads) k_seg_compact(const uint32_t* __restrict__ keys, uint32_t n,
                                                          const uint32_t* __restrict__ triOffsets, uint32_t G,
                                                          uint32_t* __restrict__ compressed,
                                                          uint32_t* __restrict__ runStarts, uint32_t* tileStatus,
                                                          uint32_t* tileCounter, uint32_t* total, uint32_t* errorWord)
{
  bc::compact_runs_tile<kThreads>(keys, n, triOffsets, G, compressed, runStarts, tileStatus, tileCounter, total,
                                  errorWord);
}

// Leaf counts and the per-geometry offsets of runs, internal nodes, LR nodes
// and records (one block; a chunked block scan over the geometries).
// counts: [0] runs (input), [1] internal nodes, [2] LR nodes, [3] records.
__global__ void __launch_bounds__(1024) k_seg_offsets(const uint32_t* __restrict__ runStarts,
                                                      const uint32_t* __restrict__ triOffsets, uint32_t G,
                                                      uint32_t* counts, uint32_t* leafOffsets, uint32_t* intOffsets,
                                                      uint32_t* nodeOffsets, uint32_t* recOffsets, BuildParams* params)
{
  const uint32_t L = counts[0];
  // first run of each geometry: the first run start >= the geometry's first triangle
  for (uint32_t s = threadIdx.x; s <= G; s += blockDim.x)
  {
    if (s == G)
    {
      leafOffsets[G] = L;
      continue;
    }
    const uint32_t t0 = triOffsets[s];
    uint32_t lo = 0, hi = L;
    while (lo < hi)
    {
      const uint32_t mid = (lo + hi) >> 1;
      if (runStarts[mid] < t0) lo = mid + 1;
      else hi = mid;
    }
    leafOffsets[s] = lo;
  }
  __syncthreads();
  __shared__ uint32_t s_carry[3];
  __shared__ uint32_t s_part[3][1024];
  if (threadIdx.x < 3) s_carry[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t base = 0; base < G; base += blockDim.x)
  {
    const uint32_t s = base + threadIdx.x;
    uint32_t a = 0, b = 0, c = 0;
    if (s < G)
    {
      const uint32_t Ls = leafOffsets[s + 1] - leafOffsets[s];
      params[s].nLeaves = Ls;
      a = Ls > 1 ? Ls - 1 : 0;             // internal nodes
      b = Ls > 0 ? 2 * Ls - 1 : 0;         // LR nodes
      c = Ls > 1 ? Ls - 1 : (Ls ? 1 : 0);  // records
    }
    s_part[0][threadIdx.x] = a;
    s_part[1][threadIdx.x] = b;
    s_part[2][threadIdx.x] = c;
    __syncthreads();
    // inclusive Hillis-Steele scan of the three columns
    for (uint32_t o = 1; o < blockDim.x; o <<= 1)
    {
      uint32_t x0 = 0, x1 = 0, x2 = 0;
      if (threadIdx.x >= o)
      {
        x0 = s_part[0][threadIdx.x - o];
        x1 = s_part[1][threadIdx.x - o];
        x2 = s_part[2][threadIdx.x - o];
      }
      __syncthreads();
      s_part[0][threadIdx.x] += x0;
      s_part[1][threadIdx.x] += x1;
      s_part[2][threadIdx.x] += x2;
      __syncthreads();
    }
    if (s < G)
    {
      intOffsets[s] = s_carry[0] + s_part[0][threadIdx.x] - a;
      nodeOffsets[s] = s_carry[1] + s_part[1][threadIdx.x] - b;
      recOffsets[s] = s_carry[2] + s_part[2][threadIdx.x] - c;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1)
    {
      s_carry[0] += s_part[0][threadIdx.x];
      s_carry[1] += s_part[1][threadIdx.x];
      s_carry[2] += s_part[2][threadIdx.x];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
  {
    intOffsets[G] = s_carry[0];
    nodeOffsets[G] = s_carry[1];
    recOffsets[G] = s_carry[2];
    counts[1] = s_carry[0];
    counts[2] = s_carry[1];
    counts[3] = s_carry[2];
  }
}

// kernel1D_MakeLeavesFromTriangles per geometry (core/builders/lbvh.cpp:350-384),
// plus the sorted triangle records and index buffer; a geometry with a single
// leaf also gets its one record (leaf + empty slot) here.
__global__ void __launch_bounds__(kThreads) k_seg_leaves(
    const float4* __restrict__ v, const uint32_t* __restrict__ idx, const uint32_t* __restrict__ vertOffsets,
    const uint32_t* __restrict__ triOffsets, const uint32_t* __restrict__ leafOffsets,
    const uint32_t* __restrict__ nodeOffsets, const uint32_t* __restrict__ recOffsets, uint32_t G,
    const uint32_t* __restrict__ counts, const uint32_t* __restrict__ sortedTri, const uint32_t* __restrict__ runStarts,
    BVHNode32* __restrict__ lr, uint32_t* __restrict__ lrCount, TriRec* __restrict__ tris,
    uint32_t* __restrict__ sortedIdx, PairRec* __restrict__ recs, uint32_t* errorWord, int vertexRecords)
{
  const uint32_t Ltot = counts[0];
  for (uint32_t g = blockIdx.x * kThreads + threadIdx.x; g < Ltot; g += gridDim.x * kThreads)
  {
    const uint32_t s = find_segment(leafOffsets, G, g);
    const uint32_t L = leafOffsets[s + 1] - leafOffsets[s];
    const uint32_t k = g - leafOffsets[s];
    const uint32_t tb = triOffsets[s], vb = vertOffsets[s], nV = vertOffsets[s + 1] - vb;
    const uint32_t start = runStarts[g];
    const uint32_t end = (k + 1 < L) ? runStarts[g + 1] : triOffsets[s + 1];
    if (k >= L || end > triOffsets[s + 1] || start >= end || start < tb)
    {
      atomicOr(errorWord, kErrLayout);
      continue;
    }
    const uint32_t count = end - start;
    if (count > 127u) atomicOr(errorWord, kErrLeafCount);
    float mn[3] = {1e10f, 1e10f, 1e10f}, mx[3] = {-1e10f, -1e10f, -1e10f};
    for (uint32_t j = start; j < end; j++)
    {
      const uint32_t tri = sortedTri[j];  // global triangle index
      uint32_t ia = idx[3 * (size_t)tri + 0], ib = idx[3 * (size_t)tri + 1], ic = idx[3 * (size_t)tri + 2];
      if (ia >= nV || ib >= nV || ic >= nV)
      {
        atomicOr(errorWord, kErrIndexRange);
        ia = ib = ic = 0;
      }
      const float4 a = v[vb + ia], b = v[vb + ib], c = v[vb + ic];
      mn[0] = lm_min(mn[0], lm_min(a.x, lm_min(b.x, c.x)));
      mn[1] = lm_min(mn[1], lm_min(a.y, lm_min(b.y, c.y)));
      mn[2] = lm_min(mn[2], lm_min(a.z, lm_min(b.z, c.z)));
      mx[0] = lm_max(mx[0], lm_max(a.x, lm_max(b.x, c.x)));
      mx[1] = lm_max(mx[1], lm_max(a.y, lm_max(b.y, c.y)));
      mx[2] = lm_max(mx[2], lm_max(a.z, lm_max(b.z, c.z)));
      TriRec r;
      r.a = make_float4(a.x, a.y, a.z, __uint_as_float(j + 1 == end ? 3u : 0u));
      r.e1 = make_float4(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y), __fsub_rn(b.z, a.z), __uint_as_float(tri - tb));
      r.e2 = make_float4(__fsub_rn(c.x, a.x), __fsub_rn(c.y, a.y), __fsub_rn(c.z, a.z), 0.0f);
      if (vertexRecords)
      {
        r.e1 = make_float4(b.x, b.y, b.z, __uint_as_float(tri - tb));
        r.e2 = make_float4(c.x, c.y, c.z, 0.0f);
      }
      tris[j] = r;
      sortedIdx[3 * (size_t)j + 0] = ia;
      sortedIdx[3 * (size_t)j + 1] = ib;
      sortedIdx[3 * (size_t)j + 2] = ic;
    }
    BVHNode32 nd;
    nd.boxMin[0] = mn[0]; nd.boxMin[1] = mn[1]; nd.boxMin[2] = mn[2];
    nd.boxMax[0] = mx[0]; nd.boxMax[1] = mx[1]; nd.boxMax[2] = mx[2];
    nd.leftOffset = pack_offset_and_size(start - tb, count);
    nd.escapeIndex = 0xFFFFFFFFu;
    lr[nodeOffsets[s] + L - 1 + k] = nd;
    lrCount[nodeOffsets[s] + L - 1 + k] = 0;
    if (L == 1u && recs != nullptr)
    {
      PairRec r;
      r.a = make_float4(mn[0], mn[1], mn[2], mx[0]);
      r.b = make_float4(mx[1], mx[2], 0.0f, 0.0f);
      r.c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      r.d = make_uint4(kLeafBit | (start - tb), kEmptyRef, 0u, 0u);
      recs[recOffsets[s]] = r;
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_seg_karras(const uint32_t* __restrict__ compressed,
                                                         const uint32_t* __restrict__ leafOffsets,
                                                         const uint32_t* __restrict__ intOffsets,
                                                         const uint32_t* __restrict__ nodeOffsets, uint32_t G,
                                                         const uint32_t* __restrict__ counts, BVHNode32* __restrict__ lr,
                                                         uint32_t* __restrict__ parent, uint32_t* __restrict__ rangeEnd)
{
  const uint32_t Itot = counts[1];
  // one node per thread; a warp's 32 consecutive internal nodes exchange
  // their codes for the direction test (lanes may belong to different
  // geometries), so the loop bound is uniform over the warp
  const uint32_t lane = threadIdx.x & 31u;
  for (uint32_t base = blockIdx.x * kThreads + (threadIdx.x & ~31u); base < Itot; base += gridDim.x * kThreads)
  {
    const uint32_t j = base + lane;
    const bool active = j < Itot;
    const uint32_t s = active ? find_segment(intOffsets, G, j) : 0u;
    const int L = active ? (int)(leafOffsets[s + 1] - leafOffsets[s]) : 0;
    const int i = active ? (int)(j - intOffsets[s]) : 0;
    uint32_t ci;
    int dPrev, dNext;
    bc::karras_neighbours(compressed, active ? (int)leafOffsets[s] : 0, L, i, active, ci, dPrev, dNext);
    if (!active) continue;
    uint32_t left, right;
    int other;
    bc::karras_node(compressed + leafOffsets[s], L, i, ci, dPrev, dNext, left, right, other);
    const uint32_t nb = nodeOffsets[s];
    lr[nb + i].leftOffset = left;
    lr[nb + i].escapeIndex = right;
    parent[nb + left] = (uint32_t)i;
    parent[nb + right] = (uint32_t)i;
    rangeEnd[j] = (uint32_t)other;
  }
}

// Bottom-up refit per geometry (as k_refit in build.cu, local numbering).
__global__ void __launch_bounds__(bc::kRefitThreads, bc::kRefitMinBlocks) k_seg_refit(const uint32_t* __restrict__ leafOffsets,
                                                        const uint32_t* __restrict__ intOffsets,
                                                        const uint32_t* __restrict__ nodeOffsets, uint32_t G,
                                                        const uint32_t* __restrict__ counts, BVHNode32* lr,
                                                        uint32_t* lrCount, const uint32_t* __restrict__ parent,
                                                        uint32_t* visit, const uint32_t* __restrict__ rangeEnd,
                                                        uint32_t* errorWord)
{
  // A block owns the global leaves [lo, hi).  Internal node p of geometry s
  // (leaf base lb) with range [a, b] lies in the slice when lb + a >= lo and
  // lb + b < hi; such nodes finish with shared-memory counters indexed by
  // lb + p (unique across geometries, inside the slice), the others with the
  // device-wide counters, as in the single-geometry refit.
  __shared__ uint32_t s_visit[bc::kRefitSlice];
  const uint32_t Ltot = counts[0];
  const uint32_t lo = blockIdx.x * bc::kRefitSlice;
  if (lo >= Ltot) return;
  const uint32_t hi = min(lo + bc::kRefitSlice, Ltot);
  for (uint32_t k = threadIdx.x; k < bc::kRefitSlice; k += bc::kRefitThreads) s_visit[k] = 0u;
  __syncthreads();
  for (uint32_t g = lo + threadIdx.x; g < hi; g += bc::kRefitThreads)
  {
    const uint32_t s = find_segment(leafOffsets, G, g);
    const uint32_t lb = leafOffsets[s];
    const uint32_t L = leafOffsets[s + 1] - lb;
    const uint32_t nb = nodeOffsets[s], ib = intOffsets[s];
    uint32_t node = L - 1 + (g - lb);
    bool inSlice = true;
    while (node != 0)
    {
      const uint32_t p = parent[nb + node];
      if (p + 1u >= L)
      {
        atomicOr(errorWord, kErrLayout);
        break;
      }
      if (inSlice)
      {
        const uint32_t j = rangeEnd[ib + p];
        inSlice = lb + (p < j ? p : j) >= lo && lb + (p > j ? p : j) < hi;
      }
      uint32_t l, r;
      float4 alo, ahi, blo, bhi;
      uint32_t cl, cr;
      if (inSlice)
      {
        if (bc::atomic_add_acq_rel_cta(&s_visit[lb + p - lo], 1u) == 0u) break;
        if (p == 0u) visit[ib] = 2u;  // the root finished inside the slice (k_seg_records checks the counter)
        l = lr[nb + p].leftOffset;
        r = lr[nb + p].escapeIndex;
        const float4* a = reinterpret_cast<const float4*>(lr + nb + l);
        const float4* b = reinterpret_cast<const float4*>(lr + nb + r);
        alo = a[0];
        ahi = a[1];
        blo = b[0];
        bhi = b[1];
        cl = lrCount[nb + l];
        cr = lrCount[nb + r];
      }
      else
      {
        if (bc::atomic_add_acq_rel(&visit[ib + p], 1u) == 0u) break;
        l = __ldcg(&lr[nb + p].leftOffset);
        r = __ldcg(&lr[nb + p].escapeIndex);
        bc::load_node_cg(lr + nb + l, alo, ahi);
        bc::load_node_cg(lr + nb + r, blo, bhi);
        cl = __ldcg(&lrCount[nb + l]);
        cr = __ldcg(&lrCount[nb + r]);
      }
      bc::store_parent(lr + nb + p, alo, ahi, blo, bhi, l, r);
      lrCount[nb + p] = cl + cr + 2u;
      node = p;
    }
  }
}

// Child-pair records per internal node (as k_records in build.cu; references
// local to the geometry: internal child -> record index, leaf -> first
// triangle of the geometry's sorted order).
__global__ void __launch_bounds__(kThreads) k_seg_records(const uint32_t* __restrict__ triOffsets,
                                                          const uint32_t* __restrict__ leafOffsets,
                                                          const uint32_t* __restrict__ intOffsets,
                                                          const uint32_t* __restrict__ nodeOffsets,
                                                          const uint32_t* __restrict__ recOffsets, uint32_t G,
                                                          const uint32_t* __restrict__ counts,
                                                          const BVHNode32* __restrict__ lr,
                                                          const uint32_t* __restrict__ runStarts,
                                                          const uint32_t* __restrict__ visit, PairRec* __restrict__ recs,
                                                          uint32_t* errorWord)
{
  if (recs == nullptr)
  {
    // 4-wide layouts keep no pair records: only the check of each root
    for (uint32_t s = blockIdx.x * kThreads + threadIdx.x; s < G; s += gridDim.x * kThreads)
      if (intOffsets[s + 1] > intOffsets[s] && visit[intOffsets[s]] != 2u) atomicOr(errorWord, kErrLayout);
    return;
  }
  const uint32_t Itot = counts[1];
  for (uint32_t j = blockIdx.x * kThreads + threadIdx.x; j < Itot; j += gridDim.x * kThreads)
  {
    const uint32_t s = find_segment(intOffsets, G, j);
    const uint32_t L = leafOffsets[s + 1] - leafOffsets[s];
    const uint32_t i = j - intOffsets[s];
    if (i == 0 && visit[j] != 2u) atomicOr(errorWord, kErrLayout);  // the refit reached this root twice
    const uint32_t nb = nodeOffsets[s], tb = triOffsets[s], lb = leafOffsets[s];
    const BVHNode32 n = lr[nb + i];
    const BVHNode32 a = lr[nb + n.leftOffset];
    const BVHNode32 b = lr[nb + n.escapeIndex];
    const uint32_t lref = (n.leftOffset < L - 1) ? n.leftOffset : (kLeafBit | (runStarts[lb + n.leftOffset - (L - 1)] - tb));
    const uint32_t rref =
        (n.escapeIndex < L - 1) ? n.escapeIndex : (kLeafBit | (runStarts[lb + n.escapeIndex - (L - 1)] - tb));
    PairRec r;
    r.a = make_float4(a.boxMin[0], a.boxMin[1], a.boxMin[2], a.boxMax[0]);
    r.b = make_float4(a.boxMax[1], a.boxMax[2], b.boxMin[0], b.boxMin[1]);
    r.c = make_float4(b.boxMin[2], b.boxMax[0], b.boxMax[1], b.boxMax[2]);
    r.d = make_uint4(lref, rref, 0u, 0u);
    recs[recOffsets[s] + i] = r;
  }
}

// Last stage: run starts and triangle ids become local to their geometry, so
// every geometry's arrays read exactly like a single build's.
__global__ void __launch_bounds__(kThreads) k_seg_localize(const uint32_t* __restrict__ triOffsets,
                                                           const uint32_t* __restrict__ leafOffsets, uint32_t G,
                                                           uint32_t N, const uint32_t* __restrict__ counts,
                                                           uint32_t* __restrict__ runStarts, uint32_t* __restrict__ vals)
{
  const uint32_t Ltot = counts[0];
  for (uint32_t t = blockIdx.x * kThreads + threadIdx.x; t < N; t += gridDim.x * kThreads)
  {
    vals[t] -= triOffsets[find_segment(triOffsets, G, t)];
    if (t < Ltot) runStarts[t] -= triOffsets[find_segment(leafOffsets, G, t)];
  }
}

inline uint32_t grid_for(uint64_t n, int numSMs, int perSM = 8)
{
  uint64_t g = (n + kThreads - 1) / kThreads;
  const uint64_t cap = (uint64_t)numSMs * perSM;
  if (g > cap) g = cap;
  return g == 0 ? 1u : (uint32_t)g;
}

inline size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

size_t build_batch_scratch_bytes(uint32_t nTris, uint32_t G)
{
  const size_t tiles = (nTris + kThreads * bc::kScanItems - 1) / (kThreads * bc::kScanItems);
  return align256(sizeof(uint32_t) * (4 + tiles)) + align256(radix_sort_segmented_scratch_bytes(nTris, G));
}

cudaError_t build_lbvh_batch(const BatchBuffers& b, int numSMs, cudaStream_t s)
{
  const uint32_t N = b.nTris, G = b.G;
  if (N == 0 || G == 0) return cudaSuccess;
  char* scratch = (char*)b.scratch;
  const size_t tiles = (N + kThreads * bc::kScanItems - 1) / (kThreads * bc::kScanItems);
  const size_t scanBytes = align256(sizeof(uint32_t) * (4 + tiles));
  uint32_t* scanCounter = (uint32_t*)scratch;
  uint32_t* scanStatus = scanCounter + 4;
  void* sortScratch = scratch + scanBytes;

  if (b.nBoxChunks) k_seg_box_partial<<<b.nBoxChunks, kThreads, 0, s>>>(b.verts, b.vertOffsets, b.boxChunkOffsets, G,
                                                                         b.boxPartial);
  k_seg_box_final<<<(G + kThreads - 1) / kThreads, kThreads, 0, s>>>(b.boxChunkOffsets, G, b.boxPartial, b.params,
                                                                      b.mortonCubic);
  k_seg_morton<<<(N + kThreads - 1) / kThreads, kThreads, 0, s>>>(b.verts, b.idx, b.vertOffsets, b.triOffsets, G, N,
                                                                   b.params, b.keys, b.vals, b.errorWord);
  cudaError_t e = cudaMemcpyAsync(b.keysUnsorted, b.keys, sizeof(uint32_t) * N, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return e;
  e = radix_sort_pairs_segmented(b.keys, b.vals, b.keysAlt, b.valsAlt, N, b.triOffsets, G, sortScratch, b.errorWord,
                                 numSMs, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(scratch, 0, scanBytes, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(b.counts, 0, 4 * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  k_seg_compact<<<(uint32_t)tiles, kThreads, 0, s>>>(b.keys, N, b.triOffsets, G, b.compressed, b.runStarts, scanStatus,
                                                    scanCounter, b.counts, b.errorWord);
  k_seg_offsets<<<1, 1024, 0, s>>>(b.runStarts, b.triOffsets, G, b.counts, b.leafOffsets, b.intOffsets, b.nodeOffsets,
                                   b.recOffsets, b.params);
  const uint32_t g = grid_for(N, numSMs, 8);
  e = cudaMemsetAsync(b.parent, 0xFF, sizeof(uint32_t) * 2 * (size_t)N, s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(b.visit, 0, sizeof(uint32_t) * N, s);
  if (e != cudaSuccess) return e;
  k_seg_leaves<<<g, kThreads, 0, s>>>(b.verts, b.idx, b.vertOffsets, b.triOffsets, b.leafOffsets, b.nodeOffsets,
                                      b.recOffsets, G, b.counts, b.vals, b.runStarts, b.lr, b.lrCount, b.tris,
                                      b.sortedIdx, b.recs, b.errorWord, b.vertexRecords);
  k_seg_karras<<<g, kThreads, 0, s>>>(b.compressed, b.leafOffsets, b.intOffsets, b.nodeOffsets, G, b.counts, b.lr,
                                      b.parent, b.visit + N);
  k_seg_refit<<<(N + bc::kRefitSlice - 1) / bc::kRefitSlice, bc::kRefitThreads, 0, s>>>(
      b.leafOffsets, b.intOffsets, b.nodeOffsets, G, b.counts, b.lr, b.lrCount, b.parent, b.visit, b.visit + N,
      b.errorWord);
  k_seg_records<<<g, kThreads, 0, s>>>(b.triOffsets, b.leafOffsets, b.intOffsets, b.nodeOffsets, b.recOffsets, G,
                                       b.counts, b.lr, b.runStarts, b.visit, b.recs, b.errorWord);
  k_seg_localize<<<g, kThreads, 0, s>>>(b.triOffsets, b.leafOffsets, G, N, b.counts, b.runStarts, b.vals);
  return cudaGetLastError();
}

}  // namespace hrt
