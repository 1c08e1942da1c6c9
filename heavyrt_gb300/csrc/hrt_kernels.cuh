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
  uint32_t*  visit;           // nTris
  PairRec*   recs;            // max(nTris-1, 1)
  TriRec*    tris;            // nTris
  uint32_t*  sortedIdx;       // 3*nTris
  BuildParams* params;        // device
  void*      scratch;         // build_scratch_bytes(nTris)
};
size_t build_scratch_bytes(uint32_t nTris);
// Runs the whole LBVH build asynchronously on `stream`.  Errors found on the
// device are ORed into params->error.
cudaError_t build_lbvh(const BuildBuffers& b, int numSMs, cudaStream_t stream);

// ---------------------------------------------------------------- trace.cu
// One instance of a geometry as the traversal sees it.
struct InstanceDesc
{
  const PairRec* recs;
  const TriRec*  tris;
  uint32_t       geomId;
  uint32_t       instId;
  uint32_t       identity;  // 1: the inverse transform is the identity, rays are used as given
  uint32_t       valid;     // 0: the geometry has no triangles
  float          inv[12];   // rows 0..2 of the inverse instance matrix (row-major)
};

struct TraceArgs
{
  const float4*       rays;       // 2 float4 per ray
  uint64_t            n;
  const InstanceDesc* inst;       // device array
  uint32_t            nInst;
  void*               hits;       // hrt_hit[n] (nearest) or uint8_t[n] (any)
  unsigned long long* counters;   // optional [2]: node pairs, triangle tests
  uint32_t*           errorWord;  // device
};
// kind 0: nearest, 1: any.  counting = 1 also accumulates counters.
cudaError_t trace(const TraceArgs& a, int kind, int counting, int numSMs, cudaStream_t stream);

}  // namespace hrt
