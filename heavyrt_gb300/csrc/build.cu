// LBVH build on the GPU: scene box, Morton codes, stable sort, run compaction,
// leaves, Karras hierarchy, atomic bottom-up refit and the 64-byte traversal
// records.  Every stage reproduces the integer and float results of HeavyRT's
// LBVHBuilder (core/builders/lbvh.cpp) bit for bit; float arithmetic is written
// with explicit round-to-nearest intrinsics so that no multiply-add is fused.
#include "build_common.cuh"
#include "hrt_kernels.cuh"

namespace hrt
{
namespace
{

constexpr int kThreads = 256;

// ---------------------------------------------------------------- scene box
// kernel1D_RedunctionFromVertices, core/builders/lbvh.cpp:228-239.  min/max
// are exact, so only the sign of a zero bound can depend on the reduction
// order; it never reaches a Morton code (+0 and -0 give the same quantised
// offset).
__global__ void __launch_bounds__(kThreads) k_box_partial(const float4* __restrict__ v, uint32_t n, float4* partial)
{
  float4 mn = make_float4(1e10f, 1e10f, 1e10f, 1e10f), mx = make_float4(-1e10f, -1e10f, -1e10f, -1e10f);
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
  {
    const float4 p = v[i];
    mn.x = lm_min(mn.x, p.x); mn.y = lm_min(mn.y, p.y); mn.z = lm_min(mn.z, p.z); mn.w = lm_min(mn.w, p.w);
    mx.x = lm_max(mx.x, p.x); mx.y = lm_max(mx.y, p.y); mx.z = lm_max(mx.z, p.z); mx.w = lm_max(mx.w, p.w);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    mn.x = lm_min(mn.x, __shfl_down_sync(0xFFFFFFFFu, mn.x, o));
    mn.y = lm_min(mn.y, __shfl_down_sync(0xFFFFFFFFu, mn.y, o));
    mn.z = lm_min(mn.z, __shfl_down_sync(0xFFFFFFFFu, mn.z, o));
    mn.w = lm_min(mn.w, __shfl_down_sync(0xFFFFFFFFu, mn.w, o));
    mx.x = lm_max(mx.x, __shfl_down_sync(0xFFFFFFFFu, mx.x, o));
    mx.y = lm_max(mx.y, __shfl_down_sync(0xFFFFFFFFu, mx.y, o));
    mx.z = lm_max(mx.z, __shfl_down_sync(0xFFFFFFFFu, mx.z, o));
    mx.w = lm_max(mx.w, __shfl_down_sync(0xFFFFFFFFu, mx.w, o));
  }
  __shared__ float4 smn[kThreads / 32], smx[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { smn[warp] = mn; smx[warp] = mx; }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    for (int w = 1; w < kThreads / 32; w++)
    {
      mn.x = lm_min(mn.x, smn[w].x); mn.y = lm_min(mn.y, smn[w].y); mn.z = lm_min(mn.z, smn[w].z); mn.w = lm_min(mn.w, smn[w].w);
      mx.x = lm_max(mx.x, smx[w].x); mx.y = lm_max(mx.y, smx[w].y); mx.z = lm_max(mx.z, smx[w].z); mx.w = lm_max(mx.w, smx[w].w);
    }
    partial[2 * blockIdx.x + 0] = mn;
    partial[2 * blockIdx.x + 1] = mx;
  }
}

// Final box and ZIndexMultCoeff on the box widened by 1e-4
// (core/builders/lbvh.cpp:41-51,263).
__global__ void __launch_bounds__(kThreads) k_box_final(const float4* __restrict__ partial, uint32_t nPartial,
                                                         BuildParams* params, int cubic)
{
  float mn[4] = {1e10f, 1e10f, 1e10f, 1e10f}, mx[4] = {-1e10f, -1e10f, -1e10f, -1e10f};
  for (uint32_t b = threadIdx.x; b < nPartial; b += kThreads)
  {
    const float4 a = partial[2 * b], c = partial[2 * b + 1];
    mn[0] = lm_min(mn[0], a.x); mn[1] = lm_min(mn[1], a.y); mn[2] = lm_min(mn[2], a.z); mn[3] = lm_min(mn[3], a.w);
    mx[0] = lm_max(mx[0], c.x); mx[1] = lm_max(mx[1], c.y); mx[2] = lm_max(mx[2], c.z); mx[3] = lm_max(mx[3], c.w);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
      mn[k] = lm_min(mn[k], __shfl_down_sync(0xFFFFFFFFu, mn[k], o));
      mx[k] = lm_max(mx[k], __shfl_down_sync(0xFFFFFFFFu, mx[k], o));
    }
  __shared__ float smn[kThreads / 32][4], smx[kThreads / 32][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int k = 0; k < 4; k++) { smn[warp][k] = mn[k]; smx[warp][k] = mx[k]; }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < kThreads / 32; w++)
    for (int k = 0; k < 4; k++) { mn[k] = lm_min(mn[k], smn[w][k]); mx[k] = lm_max(mx[k], smx[w][k]); }
  bc::zindex_scale(mn, mx, params, cubic);
}

// ---------------------------------------------------------------- Morton codes
// kernel1D_EvalMortonCodesFromTriangles, core/builders/lbvh.cpp:259-287: box
// centre (or the centroid 0.33333333*(v1+v2+v3) when fewer than 256
// triangles), quantised against the scene box with truncation toward zero.
__global__ void __launch_bounds__(kThreads) k_morton(const float4* __restrict__ v, const uint32_t* __restrict__ idx,
                                                     uint32_t nTris, uint32_t nVerts, const BuildParams* __restrict__ params,
                                                     uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                     uint32_t* errorWord)
{
  const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= nTris) return;
  uint32_t ia = idx[3 * (size_t)i + 0], ib = idx[3 * (size_t)i + 1], ic = idx[3 * (size_t)i + 2];
  if (ia >= nVerts || ib >= nVerts || ic >= nVerts)
  {
    atomicOr(errorWord, kErrIndexRange);
    ia = ib = ic = 0;
  }
  keys[i] = bc::morton_code(v[ia], v[ib], v[ic], nTris, params->bmin, params->scale);
  vals[i] = i;
}

// ---------------------------------------------------------------- run compaction
// kernel1D_AppendInit + exclusive_scan + kernel1D_AppendComplete
// (core/builders/lbvh.cpp:289-319,762-767) as one single-pass scan with
// decoupled look-back: flag = code differs from its predecessor; flagged
// positions are appended to (compressed, runStarts) in order.
using bc::kScanItems;
constexpr uint32_t kScanTile = kThreads * kScanItems;
using bc::kFlagAgg;
using bc::kFlagPrefix;
using bc::kValueMask;
using bc::kSpinLimit;
using bc::load_relaxed;
using bc::store_relaxed;

__global__ void __launch_bounds__(kThreads) k_compact_runs(const uint32_t* __restrict__ keys, uint32_t n,
                                                           uint32_t* __restrict__ compressed,
                                                           uint32_t* __restrict__ runStarts, uint32_t* tileStatus,
                                                           uint32_t* tileCounter, BuildParams* params,
                                                           uint32_t* errorWord)
{
  bc::compact_runs_tile<kThreads>(keys, n, nullptr, 0u, compressed, runStarts, tileStatus, tileCounter,
                                  &params->nLeaves, errorWord);
}

// ---------------------------------------------------------------- leaves
// kernel1D_MakeLeavesFromTriangles, core/builders/lbvh.cpp:350-384: leaf i is
// node L-1+i, its box is the union of its run's triangle boxes taken in
// sorted order.  The same loop writes the sorted triangle records and index
// buffer (AppendTreeData, core/BVH2CommonRT_host.cpp:45-64).
__global__ void __launch_bounds__(kThreads) k_leaves(const float4* __restrict__ v, const uint32_t* __restrict__ idx,
                                                     const uint32_t* __restrict__ sortedTri,
                                                     const uint32_t* __restrict__ runStarts, uint32_t nTris,
                                                     uint32_t nVerts, const BuildParams* __restrict__ params,
                                                     BVHNode32* __restrict__ lr, TriRec* __restrict__ tris,
                                                     uint32_t* __restrict__ sortedIdx, uint32_t* errorWord,
                                                     int vertexRecords)
{
  const uint32_t L = params->nLeaves <= nTris ? params->nLeaves : 0u;
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < L; i += gridDim.x * kThreads)
  {
    const uint32_t start = runStarts[i];
    uint32_t end = (i + 1 < L) ? runStarts[i + 1] : nTris;
    if (end > nTris || start >= end)
    {
      atomicOr(errorWord, kErrLayout);
      continue;
    }
    const uint32_t count = end - start;
    if (count > 127u) atomicOr(errorWord, kErrLeafCount);
    float mn[3] = {1e10f, 1e10f, 1e10f}, mx[3] = {-1e10f, -1e10f, -1e10f};
    for (uint32_t j = start; j < end; j++)
    {
      const uint32_t tri = sortedTri[j];
      uint32_t ia = idx[3 * (size_t)tri + 0], ib = idx[3 * (size_t)tri + 1], ic = idx[3 * (size_t)tri + 2];
      if (ia >= nVerts || ib >= nVerts || ic >= nVerts)
      {
        atomicOr(errorWord, kErrIndexRange);
        ia = ib = ic = 0;
      }
      const float4 a = v[ia], b = v[ib], c = v[ic];
      mn[0] = lm_min(mn[0], lm_min(a.x, lm_min(b.x, c.x)));
      mn[1] = lm_min(mn[1], lm_min(a.y, lm_min(b.y, c.y)));
      mn[2] = lm_min(mn[2], lm_min(a.z, lm_min(b.z, c.z)));
      mx[0] = lm_max(mx[0], lm_max(a.x, lm_max(b.x, c.x)));
      mx[1] = lm_max(mx[1], lm_max(a.y, lm_max(b.y, c.y)));
      mx[2] = lm_max(mx[2], lm_max(a.z, lm_max(b.z, c.z)));
      TriRec r;
      // flags: bit 0 ends a binary leaf, bit 1 a 4-wide leaf (cleared later
      // where the collapse merges two leaves)
      r.a = make_float4(a.x, a.y, a.z, __uint_as_float(j + 1 == end ? 3u : 0u));
      r.e1 = make_float4(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y), __fsub_rn(b.z, a.z), __uint_as_float(tri));
      r.e2 = make_float4(__fsub_rn(c.x, a.x), __fsub_rn(c.y, a.y), __fsub_rn(c.z, a.z), 0.0f);
      if (vertexRecords)
      {
        // the watertight test wants the vertices themselves
        r.e1 = make_float4(b.x, b.y, b.z, __uint_as_float(tri));
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
    nd.leftOffset = pack_offset_and_size(start, count);
    nd.escapeIndex = 0xFFFFFFFFu;
    lr[L - 1 + i] = nd;
  }
}

// ---------------------------------------------------------------- Karras 2012
// delta() and kernel1D_Karras12, core/builders/lbvh.cpp:386-441.  The codes
// are unique after compaction, so delta(i,j) is the count of leading zeros of
// their XOR (32 for equal codes, -1 out of range, as the reference defines).
__global__ void __launch_bounds__(kThreads) k_karras(const uint32_t* __restrict__ codes,
                                                     const BuildParams* __restrict__ params, BVHNode32* __restrict__ lr,
                                                     uint32_t* __restrict__ parent, uint32_t* __restrict__ rangeEnd)
{
  const int L = (int)params->nLeaves;
  // one node per thread; a warp's 32 consecutive nodes exchange their codes
  // for the direction test (karras_neighbours), so the loop bound is uniform
  // over the warp
  const int lane = (int)(threadIdx.x & 31u);
  for (int base = (int)(blockIdx.x * kThreads + (threadIdx.x & ~31u)); base < L - 1; base += gridDim.x * kThreads)
  {
    const int i = base + lane;
    const bool active = i < L - 1;
    uint32_t ci;
    int dPrev, dNext;
    bc::karras_neighbours(codes, 0, L, i, active, ci, dPrev, dNext);
    if (!active) continue;
    uint32_t left, right;
    int other;
    bc::karras_node(codes, L, i, ci, dPrev, dNext, left, right, other);
    lr[i].leftOffset = left;
    lr[i].escapeIndex = right;
    parent[left] = (uint32_t)i;
    parent[right] = (uint32_t)i;
    rangeEnd[i] = (uint32_t)other;
  }
}

// ---------------------------------------------------------------- refit
// Bottom-up box union.  The reference runs 32 sweeps over all internal nodes
// (core/builders/lbvh.cpp:443-489, :798-802); here each leaf walks towards the
// root and the second child to arrive at a node computes it, so every node is
// computed once from its finished children: box = (min, max) of the children
// in (left, right) order, count = children's counts + 2.
//
// A block owns the leaves [lo, hi) of one slice.  An internal node i of a
// Karras tree has i as one end of its leaf range, so the nodes whose range
// lies inside the slice are i in [lo, hi - 1): they are finished inside the
// block, with arrival counters in shared memory (acquire-release at block
// scope, children read through L1, coherent within the SM).  Only the nodes
// whose range leaves the slice use the device-wide counters (acquire-release
// at device scope, children read from L2).  Every node a thread reads was
// written by the thread that released the counter it acquired.
using bc::atomic_add_acq_rel;
using bc::atomic_add_acq_rel_cta;
using bc::kRefitSlice;

using bc::kRefitMinBlocks;
using bc::kRefitThreads;

__global__ void __launch_bounds__(kRefitThreads, kRefitMinBlocks)
    k_refit(BuildParams* params, BVHNode32* lr, uint32_t* lrCount, const uint32_t* __restrict__ parent,
            uint32_t* visit, const uint32_t* __restrict__ rangeEnd)
{
  __shared__ uint32_t s_visit[kRefitSlice];
  const uint32_t L = params->nLeaves;
  const uint32_t lo = blockIdx.x * kRefitSlice;
  if (lo >= L) return;
  const uint32_t hi = min(lo + kRefitSlice, L);
  for (uint32_t k = threadIdx.x; k < kRefitSlice; k += kRefitThreads) s_visit[k] = 0u;
  __syncthreads();
  for (uint32_t i = lo + threadIdx.x; i < hi; i += kRefitThreads)
  {
    uint32_t node = L - 1 + i;
    lrCount[node] = 0;
    bool inSlice = true;
    while (node != 0)
    {
      const uint32_t p = parent[node];
      if (p + 1u >= L)  // not an internal node: the hierarchy is inconsistent
      {
        atomicOr(&params->error, kErrLayout);
        break;
      }
      if (inSlice)
      {
        const uint32_t j = rangeEnd[p];
        inSlice = (p < j ? p : j) >= lo && (p > j ? p : j) < hi;
      }
      uint32_t l, r;
      float4 alo, ahi, blo, bhi;
      uint32_t cl, cr;
      if (inSlice)
      {
        if (atomic_add_acq_rel_cta(&s_visit[p - lo], 1u) == 0u) break;  // the sibling is not finished yet
        if (p == 0u) visit[0] = 2u;  // the root finished inside the slice (k_check_root reads the device counter)
        l = lr[p].leftOffset;
        r = lr[p].escapeIndex;
        const float4* a = reinterpret_cast<const float4*>(lr + l);
        const float4* b = reinterpret_cast<const float4*>(lr + r);
        alo = a[0];
        ahi = a[1];
        blo = b[0];
        bhi = b[1];
        cl = lrCount[l];
        cr = lrCount[r];
      }
      else
      {
        if (atomic_add_acq_rel(&visit[p], 1u) == 0u) break;
        l = __ldcg(&lr[p].leftOffset);
        r = __ldcg(&lr[p].escapeIndex);
        bc::load_node_cg(lr + l, alo, ahi);
        bc::load_node_cg(lr + r, blo, bhi);
        cl = __ldcg(&lrCount[l]);
        cr = __ldcg(&lrCount[r]);
      }
      bc::store_parent(lr + p, alo, ahi, blo, bhi, l, r);
      lrCount[p] = cl + cr + 2u;
      node = p;
    }
  }
}

// ---------------------------------------------------------------- traversal records
// One 64-byte record per internal node holding both children (the reference's
// sibling pair, core/BVH2CommonRT.cpp:91-92).  With a single leaf the record
// holds that leaf and an empty slot, as the reference pairs a lone root leaf
// with a dummy node (core/builders/lbvh.cpp:497-503, core/builders/cbvh.h:28-36).
__global__ void __launch_bounds__(kThreads) k_records(const BuildParams* __restrict__ params,
                                                      const BVHNode32* __restrict__ lr,
                                                      const uint32_t* __restrict__ runStarts, PairRec* __restrict__ recs)
{
  const uint32_t L = params->nLeaves;
  const uint32_t first = blockIdx.x * kThreads + threadIdx.x;
  if (L == 1u)
  {
    if (first == 0)
    {
      const BVHNode32 n = lr[0];
      PairRec r;
      r.a = make_float4(n.boxMin[0], n.boxMin[1], n.boxMin[2], n.boxMax[0]);
      r.b = make_float4(n.boxMax[1], n.boxMax[2], 0.0f, 0.0f);
      r.c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      r.d = make_uint4(kLeafBit | runStarts[0], kEmptyRef, 0u, 0u);
      recs[0] = r;
    }
    return;
  }
  for (uint32_t i = first; i + 1 < L; i += gridDim.x * kThreads)
  {
    const BVHNode32 n = lr[i];
    const BVHNode32 a = lr[n.leftOffset];
    const BVHNode32 b = lr[n.escapeIndex];
    const uint32_t lref = (n.leftOffset < L - 1) ? n.leftOffset : (kLeafBit | runStarts[n.leftOffset - (L - 1)]);
    const uint32_t rref = (n.escapeIndex < L - 1) ? n.escapeIndex : (kLeafBit | runStarts[n.escapeIndex - (L - 1)]);
    PairRec r;
    r.a = make_float4(a.boxMin[0], a.boxMin[1], a.boxMin[2], a.boxMax[0]);
    r.b = make_float4(a.boxMax[1], a.boxMax[2], b.boxMin[0], b.boxMin[1]);
    r.c = make_float4(b.boxMin[2], b.boxMax[0], b.boxMax[1], b.boxMax[2]);
    r.d = make_uint4(lref, rref, 0u, 0u);
    recs[i] = r;
  }
}

__global__ void k_check_root(BuildParams* params, const uint32_t* __restrict__ visit, uint32_t* errorWord)
{
  const uint32_t L = params->nLeaves;
  if (L >= 2u && visit[0] != 2u) atomicOr(errorWord, kErrLayout);
}

inline uint32_t grid_for(uint64_t n, int numSMs, int perSM = 8)
{
  uint64_t g = (n + kThreads - 1) / kThreads;
  const uint64_t cap = (uint64_t)numSMs * perSM;
  if (g > cap) g = cap;
  return g == 0 ? 1u : (uint32_t)g;
}

}  // namespace

size_t build_scratch_bytes(uint32_t nTris)
{
  const size_t partials = 2 * sizeof(float4) * 1024;
  const size_t scanTiles = (nTris + kScanTile - 1) / kScanTile;
  const size_t scan = sizeof(uint32_t) * (4 + scanTiles);
  const size_t sort = radix_sort_scratch_bytes(nTris);
  return ((partials + 255) / 256) * 256 + ((scan + 255) / 256) * 256 + sort;
}

cudaError_t build_lbvh(const BuildBuffers& b, int numSMs, cudaStream_t s)
{
  const uint32_t N = b.nTris;
  if (N == 0) return cudaSuccess;
  char* scratch = (char*)b.scratch;
  float4* partial = (float4*)scratch;
  const size_t partialBytes = ((2 * sizeof(float4) * 1024 + 255) / 256) * 256;
  uint32_t* scanCounter = (uint32_t*)(scratch + partialBytes);
  uint32_t* scanStatus = scanCounter + 4;
  const size_t scanTiles = (N + kScanTile - 1) / kScanTile;
  const size_t scanBytes = ((sizeof(uint32_t) * (4 + scanTiles) + 255) / 256) * 256;
  void* sortScratch = scratch + partialBytes + scanBytes;
  uint32_t* err = &b.params->error;

  // 1. scene box + Morton scale
  uint32_t pb = grid_for(b.nVerts, numSMs, 4);
  if (pb > 1024) pb = 1024;
  k_box_partial<<<pb, kThreads, 0, s>>>(b.verts, b.nVerts, partial);
  k_box_final<<<1, kThreads, 0, s>>>(partial, pb, b.params, b.mortonCubic);
  // 2. Morton codes
  k_morton<<<(N + kThreads - 1) / kThreads, kThreads, 0, s>>>(b.verts, b.idx, N, b.nVerts, b.params, b.keys, b.vals, err);
  cudaError_t e = cudaMemcpyAsync(b.keysUnsorted, b.keys, sizeof(uint32_t) * N, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return e;
  // 3. stable sort by code
  e = radix_sort_pairs(b.keys, b.vals, b.keysAlt, b.valsAlt, N, sortScratch, err, numSMs, s);
  if (e != cudaSuccess) return e;
  // 4. unique codes and run starts
  e = cudaMemsetAsync(scanCounter, 0, scanBytes, s);
  if (e != cudaSuccess) return e;
  k_compact_runs<<<(uint32_t)scanTiles, kThreads, 0, s>>>(b.keys, N, b.compressed, b.runStarts, scanStatus, scanCounter,
                                                          b.params, err);
  // 5. leaves, 6. hierarchy, 7. refit, 8. records
  const uint32_t g = grid_for(N, numSMs, 8);
  k_leaves<<<g, kThreads, 0, s>>>(b.verts, b.idx, b.vals, b.runStarts, N, b.nVerts, b.params, b.lr, b.tris, b.sortedIdx, err,
                                  b.vertexRecords);
  e = cudaMemsetAsync(b.parent, 0xFF, sizeof(uint32_t) * (2 * (size_t)N - 1), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(b.visit, 0, sizeof(uint32_t) * N, s);
  if (e != cudaSuccess) return e;
  k_karras<<<g, kThreads, 0, s>>>(b.compressed, b.params, b.lr, b.parent, b.visit + N);
  k_refit<<<(N + kRefitSlice - 1) / kRefitSlice, kRefitThreads, 0, s>>>(b.params, b.lr, b.lrCount, b.parent, b.visit,
                                                                   b.visit + N);
  k_check_root<<<1, 1, 0, s>>>(b.params, b.visit, err);
  if (b.recs) k_records<<<g, kThreads, 0, s>>>(b.params, b.lr, b.runStarts, b.recs);
  return cudaGetLastError();
}

// Refit: the geometry's vertices moved, its triangles and their sorted order
// did not.  Leaves, triangle records and the sorted index buffer are rewritten
// from the new vertices in the existing order, the hierarchy's parent links are
// recomputed from the unchanged codes, and the boxes refit bottom-up; the
// Morton frame in params stays that of the build.  The geometry's new vertex
// box goes to boxOut (bmin/bmax).
cudaError_t refit_lbvh(const BuildBuffers& b, BuildParams* boxOut, int numSMs, cudaStream_t s)
{
  const uint32_t N = b.nTris;
  if (N == 0) return cudaSuccess;
  float4* partial = (float4*)b.scratch;  // refit_scratch_bytes()
  uint32_t* err = &b.params->error;
  uint32_t pb = grid_for(b.nVerts, numSMs, 4);
  if (pb > 1024) pb = 1024;
  k_box_partial<<<pb, kThreads, 0, s>>>(b.verts, b.nVerts, partial);
  k_box_final<<<1, kThreads, 0, s>>>(partial, pb, boxOut, b.mortonCubic);
  const uint32_t g = grid_for(N, numSMs, 8);
  k_leaves<<<g, kThreads, 0, s>>>(b.verts, b.idx, b.vals, b.runStarts, N, b.nVerts, b.params, b.lr, b.tris, b.sortedIdx,
                                  err, b.vertexRecords);
  cudaError_t e = cudaMemsetAsync(b.parent, 0xFF, sizeof(uint32_t) * (2 * (size_t)N - 1), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(b.visit, 0, sizeof(uint32_t) * N, s);
  if (e != cudaSuccess) return e;
  k_karras<<<g, kThreads, 0, s>>>(b.compressed, b.params, b.lr, b.parent, b.visit + N);
  k_refit<<<(N + kRefitSlice - 1) / kRefitSlice, kRefitThreads, 0, s>>>(b.params, b.lr, b.lrCount, b.parent, b.visit,
                                                                   b.visit + N);
  k_check_root<<<1, 1, 0, s>>>(b.params, b.visit, err);
  if (b.recs) k_records<<<g, kThreads, 0, s>>>(b.params, b.lr, b.runStarts, b.recs);
  return cudaGetLastError();
}

size_t refit_scratch_bytes() { return 2 * sizeof(float4) * 1024; }

}  // namespace hrt
