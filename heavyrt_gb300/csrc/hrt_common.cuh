// Shared device-side definitions of the GB300 ray-query engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hrt
{

constexpr uint32_t kLeafBit   = 0x80000000u;  // leaf marker in node words (core/raytrace_common.h:41)
constexpr uint32_t kStartMask = 0x00FFFFFFu;  // core/raytrace_common.h:38
constexpr uint32_t kSizeMask  = 0x7F000000u;  // core/raytrace_common.h:40
constexpr uint32_t kEmptyRef  = 0xFFFFFFFFu;  // child slot with no triangles (L == 1 padding)

// Device error word bits (ORed by kernels, read by the host after a build or
// a counted query).
constexpr uint32_t kErrIndexRange  = 1u << 0;  // a triangle index >= vertex count
constexpr uint32_t kErrLeafCount   = 1u << 1;  // more than 127 triangles share one Morton code
constexpr uint32_t kErrWaitTimeout = 1u << 2;  // a decoupled look-back wait gave up
constexpr uint32_t kErrStack       = 1u << 3;  // traversal stack bound exceeded
constexpr uint32_t kErrLayout      = 1u << 4;  // inconsistent tree (refit did not reach the root)
constexpr uint32_t kErrStepBudget  = 1u << 5;  // a ray exceeded its traversal step budget (ended as a miss)

// HeavyRT's BVHNode (core/builders/cbvh.h:20-26): 32 bytes, the layout of the
// LR tree the builder exports for parity checks.
struct BVHNode32
{
  float    boxMin[3];
  uint32_t leftOffset;
  float    boxMax[3];
  uint32_t escapeIndex;
};
static_assert(sizeof(BVHNode32) == 32, "BVHNode32 must be 32 bytes");

// Traversal record of one internal node: the boxes of both children and their
// references, 64 bytes = four 128-bit loads.  This is the same information as
// the reference's sibling pair nodes[o], nodes[o+1] (core/BVH2CommonRT.cpp:91-92).
//   a = (L.min.x, L.min.y, L.min.z, L.max.x)
//   b = (L.max.y, L.max.z, R.min.x, R.min.y)
//   c = (R.min.z, R.max.x, R.max.y, R.max.z)
//   d = (Lref, Rref, 0, 0)
// ref: internal child -> its record index; leaf -> kLeafBit | first sorted
// triangle; kEmptyRef -> no triangles.
struct __align__(16) PairRec
{
  float4 a, b, c;
  uint4  d;
};
static_assert(sizeof(PairRec) == 64, "PairRec must be 64 bytes");

// Triangle record in Morton-sorted order: vertex A and the two edges
// e1 = B - A, e2 = C - A (the same float subtractions the reference performs
// per test, core/BVH2CommonRT.cpp:26-27).  a.w holds flags (bit 0: last
// triangle of its leaf), e1.w the original triangle index, both as raw bits.
struct __align__(16) TriRec
{
  float4 a, e1, e2;
};
static_assert(sizeof(TriRec) == 48, "TriRec must be 48 bytes");

// 4-wide nodes (children in slots 0..3; ref as in PairRec, kEmptyRef = unused
// slot).  A leaf slot's triangles end at the record whose flags have bit 1 set.
// FP32 boxes, 128 bytes: component vectors over the four slots.
struct __align__(16) Node4F32
{
  float4 lox, loy, loz, hix, hiy, hiz;
  uint4  ref;
  uint4  pad;
};
static_assert(sizeof(Node4F32) == 128, "Node4F32 must be 128 bytes");

// FP16 boxes rounded outward, 64 bytes: a[k] = half2(lo.x, lo.y), b[k] =
// half2(lo.z, hi.x), c[k] = half2(hi.y, hi.z) for slot k.
struct __align__(16) Node4F16
{
  uint4 a, b, c, ref;
};
static_assert(sizeof(Node4F16) == 64, "Node4F16 must be 64 bytes");

// 8-bit boxes against a per-node frame, 64 bytes: frame.xyz = origin, frame.w
// = three biased exponents (e + 128, one byte per axis); bound = origin +
// q * 2^e.  q0 = bytes (lo.x, lo.y, lo.z, hi.x) per slot (slot k in byte k),
// q1.x/q1.y = (hi.y, hi.z).
struct __align__(16) Node4Q8
{
  float4 frame;
  uint4  q0, q1, ref;
};
static_assert(sizeof(Node4Q8) == 64, "Node4Q8 must be 64 bytes");

// Scene box, Morton scale and leaf count of one geometry, written on the device.
struct BuildParams
{
  float    bmin[4];
  float    bmax[4];
  float    scale[4];
  uint32_t nLeaves;
  uint32_t error;
  uint32_t rootRecord;
  uint32_t pad;
};

// LiteMath-style component min/max used for every box in the builder
// (core/builders/lbvh.cpp:220-221,374-378,475-476): returns b on ties.
__device__ __forceinline__ float lm_min(float a, float b) { return (a < b) ? a : b; }
__device__ __forceinline__ float lm_max(float a, float b) { return (a > b) ? a : b; }
// std::min / std::max as the slab test uses them (core/raytrace_common.h:72-75).
__device__ __forceinline__ float std_min(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float std_max(float a, float b) { return (a < b) ? b : a; }

__device__ __forceinline__ uint32_t pack_offset_and_size(uint32_t start, uint32_t size)
{
  return kLeafBit | ((size << 24) & kSizeMask) | (start & kStartMask);  // core/raytrace_common.h:48-51
}

}  // namespace hrt
