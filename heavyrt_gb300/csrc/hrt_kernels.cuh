// Host-side launchers of the engine's kernels (one translation unit each).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "hrt_common.cuh"

namespace hrt
{

// ---------------------------------------------------------------- radix_sort.cu
// Stable LSD onesweep radix sort of (key, value) pairs by 32-bit key, four
// 8-bit digit passes.  keys/vals hold the input and receive the output;
// keysAlt/valsAlt are ping-pong buffers of n entries.  scratch must hold
// radix_sort_scratch_bytes(n) bytes; it is cleared by the call.
constexpr uint32_t kTileSize = 4096;  // pairs per onesweep tile
size_t radix_sort_scratch_bytes(uint32_t n);
cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keysAlt, uint32_t* valsAlt, uint32_t n,
                             void* scratch, uint32_t* errorWord, int numSMs, cudaStream_t stream);
// Stable sort by (segment, key) where the segment of a pair is the segment of
// its value in segOffsets[0..segCount] (device, ascending, offsets[0] = 0):
// each segment ends up sorted by key in place of its input range.
size_t radix_sort_segmented_scratch_bytes(uint32_t n, uint32_t segCount);
cudaError_t radix_sort_pairs_segmented(uint32_t* keys, uint32_t* vals, uint32_t* keysAlt, uint32_t* valsAlt,
                                       uint32_t n, const uint32_t* segOffsets, uint32_t segCount, void* scratch,
                                       uint32_t* errorWord, int numSMs, cudaStream_t stream);

// ---------------------------------------------------------------- build.cu
struct BuildBuffers
{
  // inputs (device)
  const float4*   verts;      // nVerts, w = 1
  const uint32_t* idx;        // 3 * nTris
  uint32_t        nVerts;
  uint32_t        nTris;
  // stage arrays (device)
  uint32_t*  keys;            // nTris: Morton codes, sorted in place
  uint32_t*  vals;            // nTris: triangle ids, sorted in place
  uint32_t*  keysAlt;         // nTris: sort ping-pong
  uint32_t*  valsAlt;         // nTris
  uint32_t*  keysUnsorted;    // nTris: copy of the codes before the sort (export)
  uint32_t*  compressed;      // nTris (L used): unique codes
  uint32_t*  runStarts;       // nTris (L used)
  BVHNode32* lr;              // 2*nTris-1 (2L-1 used): Karras + refit tree
  uint32_t*  lrCount;         // 2*nTris-1
  uint32_t*  parent;          // 2*nTris-1
  uint32_t*  visit;           // 2*nTris: refit counters, then each internal node's range end
  PairRec*   recs;            // max(nTris-1, 1); null: no pair records (4-wide layouts)
  TriRec*    tris;            // nTris
  uint32_t*  sortedIdx;       // 3*nTris
  BuildParams* params;        // device
  void*      scratch;         // build_scratch_bytes(nTris)
  int        vertexRecords = 0;  // 1: triangle records hold {A, B, C} (watertight test), else {A, B-A, C-A}
  int        mortonCubic = 0;    // 1: one Morton scale for x, y, z (that of the longest axis)
};
size_t build_scratch_bytes(uint32_t nTris);
// Runs the whole LBVH build asynchronously on `stream`.  Errors found on the
// device are ORed into params->error.
cudaError_t build_lbvh(const BuildBuffers& b, int numSMs, cudaStream_t stream);
// Refit of a built LBVH after its vertices moved (same triangles, same sorted
// order): leaves, triangle records, hierarchy links, boxes and records are
// recomputed; keys, codes and runs are kept.  Uses b.verts, b.idx, b.nVerts,
// b.nTris, b.vals, b.compressed, b.runStarts, b.lr, b.lrCount, b.parent,
// b.visit, b.recs, b.tris, b.sortedIdx, b.params and b.scratch
// (refit_scratch_bytes()); the new vertex box is written to boxOut.
size_t refit_scratch_bytes();
cudaError_t refit_lbvh(const BuildBuffers& b, BuildParams* boxOut, int numSMs, cudaStream_t stream);

// ---------------------------------------------------------------- build_batch.cu
// G geometries built together.  Geometry s owns vertices
// [vertOffsets[s], vertOffsets[s+1]) and triangles [triOffsets[s],
// triOffsets[s+1]) of the concatenated inputs (indices local to its vertices).
// Its results sit at its own offsets: triangle arrays at triOffsets[s], runs at
// leafOffsets[s], LR nodes / parents at nodeOffsets[s], refit counters at
// intOffsets[s], records at recOffsets[s]; all offsets (G+1 entries) and the
// totals in counts ([0] runs, [1] internal nodes, [2] LR nodes, [3] records)
// are computed on the device.
struct BatchBuffers
{
  const float4*   verts;        // total vertices, w = 1
  const uint32_t* idx;          // 3 * nTris, local to each geometry
  const uint32_t* vertOffsets;  // G+1 (device)
  const uint32_t* triOffsets;   // G+1 (device)
  uint32_t        G;
  uint32_t        nTris;        // triOffsets[G]
  uint32_t*  keys;              // nTris
  uint32_t*  vals;              // nTris: global triangle ids in sorted order
  uint32_t*  keysAlt;           // nTris
  uint32_t*  valsAlt;           // nTris
  uint32_t*  keysUnsorted;      // nTris
  uint32_t*  compressed;        // nTris
  uint32_t*  runStarts;         // nTris: global positions
  BVHNode32* lr;                // 2*nTris
  uint32_t*  lrCount;           // 2*nTris
  uint32_t*  parent;            // 2*nTris
  uint32_t*  visit;             // 2*nTris: refit counters, then each internal node's range end
  PairRec*   recs;              // nTris; null: no pair records (4-wide layouts)
  TriRec*    tris;              // nTris; e1.w = triangle id local to the geometry
  uint32_t*  sortedIdx;         // 3*nTris, local vertex ids
  BuildParams* params;          // G: box, scale, nLeaves per geometry
  uint32_t*  leafOffsets;       // G+1
  uint32_t*  intOffsets;        // G+1
  uint32_t*  nodeOffsets;       // G+1
  uint32_t*  recOffsets;        // G+1
  uint32_t*  counts;            // 4
  uint32_t*  errorWord;         // device word shared by the batch
  void*      scratch;           // build_batch_scratch_bytes(nTris, G)
  // scene boxes: geometry s's vertices in chunks [boxChunkOffsets[s], boxChunkOffsets[s+1])
  // of kBatchBoxChunk vertices, one (min, max) float4 pair per chunk in boxPartial
  const uint32_t* boxChunkOffsets;  // G+1 (device)
  uint32_t        nBoxChunks;
  float4*         boxPartial;       // 2 * nBoxChunks
  int             vertexRecords = 0;  // as BuildBuffers::vertexRecords
  int             mortonCubic = 0;    // as BuildBuffers::mortonCubic
};
constexpr uint32_t kBatchBoxChunk = 8192;
size_t build_batch_scratch_bytes(uint32_t nTris, uint32_t G);
cudaError_t build_lbvh_batch(const BatchBuffers& b, int numSMs, cudaStream_t stream);

// ---------------------------------------------------------------- bvh4.cu
// Collapse of a finished LBVH (LR tree, parents, run starts) into 4-wide nodes.
struct Bvh4Buffers
{
  uint32_t         nTris;
  BuildParams*     params;          // device; nLeaves and the error word
  const BVHNode32* lr;              // 2L-1
  const uint32_t*  runStarts;       // L
  const uint32_t*  parent;          // 2L-1
  TriRec*          tris;            // N; bit 1 of a.w marks 4-wide leaf ends
  const uint32_t*  lrCount;         // 2L-1 descendant node counts (the largest-first collapse opens by them)
  int              mergeMode;       // 0: merge two leaf children (reference rule); M > 0: merge subtrees of <= M triangles
  int              collapse;        // HRT_BVH4_COLLAPSE_*
  void*            scratch;         // bvh4_scratch_bytes(nTris)
  uint32_t*        hostNodeCount;   // host word receiving the node count (0 when L == 1)
};
size_t bvh4_scratch_bytes(uint32_t nTris);
// Roles, depths and node numbering; copies the node count to *hostNodeCount
// (asynchronously: synchronise before reading it).
cudaError_t bvh4_plan(const Bvh4Buffers& b, int numSMs, cudaStream_t stream);
// Writes the nodes in `format` (0 FP32, 1 FP16, 2 8-bit) to `nodes`, which
// holds maxNodes nodes (the planned count).
cudaError_t bvh4_emit(const Bvh4Buffers& b, int format, void* nodes, uint32_t maxNodes, int numSMs,
                      cudaStream_t stream);

// The collapse of every geometry of a segmented build at once (device arrays
// as in BatchBuffers; runStarts local to each geometry).  bvh4_plan_batch
// copies each geometry's 4-wide node count (G words) and node offset in the
// batch's node array (G + 1 words; the last is the total) to host memory
// (asynchronously: synchronise before reading); bvh4_emit_batch writes all
// nodes, geometry s from node node4Off[s] on, numbered from its root.
struct Bvh4Batch
{
  uint32_t         G;
  const BVHNode32* lr;
  const uint32_t*  runStarts;
  const uint32_t*  parent;
  TriRec*          tris;
  const uint32_t*  leafOffsets;
  const uint32_t*  intOffsets;
  const uint32_t*  nodeOffsets;
  const uint32_t*  triOffsets;
  const uint32_t*  lrCount;  // indexed like lr
  int              mergeMode;
  int              collapse;  // HRT_BVH4_COLLAPSE_*
};
size_t bvh4_batch_scratch_bytes(uint32_t nInt, uint32_t G);
cudaError_t bvh4_plan_batch(const Bvh4Batch& b, uint32_t nInt, void* scratch, uint32_t* hostCount4,
                            uint32_t* hostNode4Off, uint32_t* errorWord, int numSMs, cudaStream_t stream);
cudaError_t bvh4_emit_batch(const Bvh4Batch& b, uint32_t nInt, void* scratch, int format, void* nodes,
                            uint32_t* errorWord, int numSMs, cudaStream_t stream);

// ---------------------------------------------------------------- trace.cu
// One instance of a geometry as the traversal sees it.
struct InstanceDesc
{
  const PairRec* recs;      // binary records (layout 0)
  const void*    nodes4;    // 4-wide nodes (layouts 1-3)
  const TriRec*  tris;
  uint32_t       geomId;
  uint32_t       instId;
  uint32_t       identity;  // 1: the inverse transform is the identity, rays are used as given
  uint32_t       valid;     // 0: the geometry has no triangles
  float          inv[12];   // rows 0..2 of the inverse instance matrix (row-major)
};

struct TraceArgs
{
  const float4*       rays;        // 2 float4 per ray
  uint64_t            n;
  const InstanceDesc* inst;        // device array
  uint32_t            nInst;
  void*               hits;        // hrt_hit[n] (nearest) or uint8_t[n] (any)
  unsigned long long* counters;    // optional [2]: node pairs, triangle tests
  uint32_t*           errorWord;   // device
  unsigned int*       rayCounter;  // device, work counter of the persistent pool
  // segmented query (optional): rays [rayOffsets[k], rayOffsets[k+1]) are
  // traced against instance segInst[k] only; device arrays of nSeg+1 / nSeg
  const uint32_t*     rayOffsets = nullptr;
  const uint32_t*     segInst = nullptr;
  uint32_t            nSeg = 0;
  // instance tree (optional): binary LBVH over the instances' world boxes;
  // its triangle records' e1.w hold instance ids
  const PairRec*      tlasRecs = nullptr;
  const TriRec*       tlasTris = nullptr;
  // host copy of the descriptor when the scene is one valid instance under the
  // identity transform (the single-instance kernel), else null
  const InstanceDesc* one = nullptr;
  // triangle test of every geometry traced: 0 Moller-Trumbore (records
  // {A, B-A, C-A}), 1 watertight (records {A, B, C})
  int                 triTest = 0;
  // L2 access-policy window of the single-instance kernels (bytes = 0: none):
  // this range of the node array is marked persisting in L2
  const void*         persistBase = nullptr;
  size_t              persistBytes = 0;
  float               persistHitRatio = 1.0f;
};

// Launch shape of the traversal (tuned per workload).
struct TraceConfig
{
  int threadsPerBlock = 128;  // 64, 128 or 256
  int persistent = 1;         // 1: persistent warp pool with lane refill; 0: one thread per ray
  int stepsPerRefill = 16;    // traversal steps between refill checks
  int refillLanes = 24;       // a warp refills when at least this many lanes are idle
  int stackEntries = 0;       // stack entries per lane in shared memory, the rest in local
                              // memory; 0 (or at least the depth bound): all in shared memory
  int imageWidth = 0;         // > 0: rays form row-major images this wide, traced in 4 x 8 tiles
};

// kind 0: nearest, 1: any.  counting = 1 also accumulates counters (node
// fetches, triangle tests).  layout: 0 binary pair records, 1 4-wide FP32,
// 2 4-wide FP16, 3 4-wide 8-bit.
cudaError_t trace(const TraceArgs& a, int kind, int counting, int layout, const TraceConfig& c, int numSMs,
                  cudaStream_t stream);

}  // namespace hrt
