// Nearest-hit / any-hit traversal of the LBVH.
//
// Each ray makes the decisions of HeavyRT's BVH2TraverseC32
// (core/BVH2CommonRT.cpp:49-141) on the same binary tree: load the two
// children of the current node, slab-test both (core/raytrace_common.h:67-80),
// descend into the nearer hit child (child 0 on equal entry distance), push
// the other, pop when neither is hit.  The leaf test is the reference's
// Moller-Trumbore with 1e-6 barycentric slack (core/BVH2CommonRT.cpp:9-47),
// written with explicit round-to-nearest intrinsics in the reference's
// evaluation order, so t/u/v match the CPU reference bit for bit.
//
// Slab distances only feed comparisons (hit tests, near-first choice, pruning
// against the current t), so the slab test takes min/max with the hardware
// fminf/fmaxf instead of the reference's std::min/std::max selects: the two
// differ only in the sign of a zero result (and for NaN, which finite rays
// never produce because SafeInverse keeps |1/d| <= 1e36), and +0 == -0 in
// every comparison, so every decision is unchanged.
//
// Scheduling: a persistent warp pool.  Each warp keeps one ray per lane; when
// enough lanes have finished, the warp refills them from a global ray counter
// with one atomic per warp (ballot + popc ranking), so lanes do not idle while
// the warp's longest ray finishes.  A ray's own visit order does not depend on
// the schedule.  A one-thread-per-ray grid is kept as a configuration.
//
// Memory: a child pair is one 64-byte record (four 128-bit read-only loads), a
// triangle one 48-byte record (three).  The stack's first S entries live in
// shared memory, interleaved by thread so a warp's pushes and pops hit 32
// different banks; deeper entries spill to a per-thread array in local memory
// (S is a launch parameter, full depth by default, so no entry spills).
//
// Triangle test: the reference's Moller-Trumbore (records {A, B-A, C-A}), or,
// for scenes built for it, the watertight test of Woop, Benthin & Wald
// (records {A, B, C}); both are template variants of the same kernels.
#pragma once

#include <cuda_fp16.h>

#include "hrt_kernels.cuh"
#include "../../include/hrt.h"

namespace hrt
{
namespace
{

// Stack bounds: the binary tree of distinct 30-bit codes is at most 30 levels
// deep (each level lengthens the common prefix), one push per level; the
// 4-wide tree halves the levels and pushes at most 3 per level.
constexpr int      kStack2 = 32;
constexpr int      kStack4 = 48;
constexpr uint32_t kNoRay = 0xFFFFFFFFu;

// With a TLAS the instance tree's entries sit below the geometry's on the
// same stack (at most kStack2 of them: the TLAS is a binary LBVH).
template <int LAYOUT, bool TLAS = false> struct StackDepth
{
  static constexpr int value = (LAYOUT == 0 ? kStack2 : kStack4) + (TLAS ? kStack2 : 0);
};

constexpr uint32_t kTlasMode = 0xFFFFFFFEu;  // Lane::inst while the lane walks the instance tree

// Order in which a launch takes its rays.  With width > 0 the rays form
// row-major images `width` rays wide, and work item i maps to a pixel of a
// tile 4 pixels wide and 8 tall (32 consecutive work items = one warp = one
// tile, tiles row after row): neighbouring pixels trace together.  Index
// arithmetic only; each ray's result still goes to the ray's own index.  (Of
// 32 x 1, 16 x 2, 8 x 4, 8 x 8 and 4 x 8 tiles, 4 x 8 traced the 1920 x 1080
// frame's eye rays fastest.)
struct RayOrder
{
  uint32_t nWork;        // work items (>= rays; tiles that cross the image edge pad it)
  uint32_t width;        // 0: work item i is ray i
  uint32_t tilesPerRow;
};

__device__ __forceinline__ uint32_t work_ray(const RayOrder& o, uint32_t i, uint32_t n)
{
  if (o.width == 0) return i < n ? i : kNoRay;
  const uint32_t t = i >> 5, l = i & 31u;
  const uint32_t x = (t % o.tilesPerRow) * 4u + (l & 3u);
  const uint32_t y = (t / o.tilesPerRow) * 8u + (l >> 2);
  if (x >= o.width) return kNoRay;
  const uint64_t r = (uint64_t)y * o.width + x;
  return r < n ? (uint32_t)r : kNoRay;
}

__host__ __forceinline__ RayOrder ray_order(uint32_t n, int width)
{
  RayOrder o{n, 0u, 0u};
  if (width <= 0 || n == 0) return o;
  const uint64_t w = (uint64_t)width;
  const uint64_t tilesPerRow = (w + 3) / 4, rows = (n + w - 1) / w;
  const uint64_t work = tilesPerRow * ((rows + 7) / 8) * 32;
  if (work > 0x7FFFFFFFull) return o;  // too much padding for 32-bit work counters: rays in order
  o.nWork = (uint32_t)work;
  o.width = (uint32_t)w;
  o.tilesPerRow = (uint32_t)tilesPerRow;
  return o;
}

// A lane's traversal stack: entries below `shared` in shared memory (entry k
// of thread t at sh[k * THREADS]), the rest in the lane's spill array.  The
// kernels without spill (SPILL = false: the whole depth bound in shared
// memory) keep the plain shared-memory addressing.
template <int THREADS, bool SPILL> struct Stack
{
  uint32_t* sh;
  uint32_t* spill;  // DEPTH - shared entries (local memory); unused without SPILL
  int       shared;
  __device__ __forceinline__ void put(int k, uint32_t v)
  {
    if (!SPILL || k < shared) sh[k * THREADS] = v;
    else spill[k - shared] = v;
  }
  __device__ __forceinline__ uint32_t get(int k) const
  {
    return (!SPILL || k < shared) ? sh[k * THREADS] : spill[k - shared];
  }
};

// Shared-memory entries per lane for a requested short-stack size (0 or
// anything at or above the depth bound: the whole stack).
template <int DEPTH> __host__ __device__ __forceinline__ int shared_entries(int requested)
{
  return (requested <= 0 || requested >= DEPTH) ? DEPTH : requested;
}

// Instance tree (TLAS): a binary LBVH over the instances' world-space boxes,
// built like a geometry's tree from one pseudo-triangle per instance; a leaf
// is a run of sorted records whose e1.w holds the instance id.
struct Tlas
{
  const PairRec* recs;  // nullptr: no TLAS, instances are taken in order
  const TriRec*  tris;
  uint32_t       nInst;
};

struct WtRay
{
  int   kx, ky, kz;
  float sx, sy, sz;
};

__device__ __forceinline__ float pick3(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ __forceinline__ void wt_setup(float dx, float dy, float dz, WtRay& w)
{
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  w.kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
  w.kx = w.kz == 2 ? 0 : w.kz + 1;
  w.ky = w.kx == 2 ? 0 : w.kx + 1;
  const float dk = pick3(dx, dy, dz, w.kz);
  if (dk < 0.0f)
  {
    const int t = w.kx;
    w.kx = w.ky;
    w.ky = t;
  }
  w.sx = __fdiv_rn(pick3(dx, dy, dz, w.kx), dk);
  w.sy = __fdiv_rn(pick3(dx, dy, dz, w.ky), dk);
  w.sz = __frcp_rn(dk);  // correctly rounded: the value of 1.0f / dk
}

// A ray in the frame of the geometry being traversed.  `w` is the watertight
// test's per-ray set-up; the Moller-Trumbore kernels never read it, so the
// compiler drops its computation there.
struct Ray
{
  float ox, oy, oz, tNear;
  float dx, dy, dz;
  float ix, iy, iz;
  WtRay w;
};


// SafeInverse, core/raytrace_common.h:57-65.
__device__ __forceinline__ float safe_inv(float d)
{
  const float ooeps = 1.0e-36f;
  return __frcp_rn(fabsf(d) > ooeps ? d : copysignf(ooeps, d));  // correctly rounded, as 1.0f / d
}

// RayBoxIntersection2, core/raytrace_common.h:67-80 (differences, products and
// evaluation order of the reference; min/max as explained above).
__device__ __forceinline__ void slab(const Ray& r, float bx0, float by0, float bz0, float bx1, float by1, float bz1,
                                     float& tn, float& tf)
{
  const float lo = __fmul_rn(r.ix, __fsub_rn(bx0, r.ox));
  const float hi = __fmul_rn(r.ix, __fsub_rn(bx1, r.ox));
  const float lo1 = __fmul_rn(r.iy, __fsub_rn(by0, r.oy));
  const float hi1 = __fmul_rn(r.iy, __fsub_rn(by1, r.oy));
  const float lo2 = __fmul_rn(r.iz, __fsub_rn(bz0, r.oz));
  const float hi2 = __fmul_rn(r.iz, __fsub_rn(bz1, r.oz));
  tn = fmaxf(fmaxf(fminf(lo, hi), fminf(lo1, hi1)), fminf(lo2, hi2));
  tf = fminf(fminf(fmaxf(lo, hi), fmaxf(lo1, hi1)), fmaxf(lo2, hi2));
}

// A 32-byte ray or hit record: one 256-bit access when the record is 32-byte
// aligned (sm_100 and later), else two 128-bit ones.  A warp's 32 records are
// then one contiguous kilobyte per instruction, which matters most for arrays
// read and written in place over the host link.
__device__ __forceinline__ void load_record(const float4* __restrict__ p, float4& a, float4& b)
{
  if ((reinterpret_cast<uintptr_t>(p) & 31u) == 0u)
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
  else
  {
    a = __ldg(p);
    b = __ldg(p + 1);
  }
}

__device__ __forceinline__ void store_record(float4* p, const float4& a, const float4& b)
{
  if ((reinterpret_cast<uintptr_t>(p) & 31u) == 0u)
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(a.x), "f"(a.y), "f"(a.z),
                 "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
                 : "memory");
  else
  {
    p[0] = a;
    p[1] = b;
  }
}

struct Hit
{
  float    t, u, v;
  uint32_t prim, inst;  // sorted triangle, instance index (0xFFFFFFFF: no hit)
};

// matmul4x3 / matmul3x3 (core/raytrace_common.h:82-90) with the column sum
// order ((m0*x + m1*y) + m2*z) + m3*w.
__device__ __forceinline__ float row_dot(const float* m, float x, float y, float z, float w)
{
  return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], x), __fmul_rn(m[1], y)), __fmul_rn(m[2], z)), __fmul_rn(m[3], w));
}

__device__ __forceinline__ void make_ray(const InstanceDesc& d, const float4& po, const float4& di, Ray& r)
{
  r.tNear = po.w;
  if (d.identity)
  {
    r.ox = po.x; r.oy = po.y; r.oz = po.z;
    r.dx = di.x; r.dy = di.y; r.dz = di.z;
  }
  else
  {
    r.ox = row_dot(d.inv + 0, po.x, po.y, po.z, 1.0f);
    r.oy = row_dot(d.inv + 4, po.x, po.y, po.z, 1.0f);
    r.oz = row_dot(d.inv + 8, po.x, po.y, po.z, 1.0f);
    r.dx = row_dot(d.inv + 0, di.x, di.y, di.z, 0.0f);
    r.dy = row_dot(d.inv + 4, di.x, di.y, di.z, 0.0f);
    r.dz = row_dot(d.inv + 8, di.x, di.y, di.z, 0.0f);
  }
  r.ix = safe_inv(r.dx);
  r.iy = safe_inv(r.dy);
  r.iz = safe_inv(r.dz);
  wt_setup(r.dx, r.dy, r.dz, r.w);
}

// Moller-Trumbore leaf test over the leaf starting at sorted triangle j
// (IntersectAllPrimitivesInLeaf, core/BVH2CommonRT.cpp:9-47); the leaf ends at
// the record whose flags have ENDBIT set (1: binary leaf, 2: 4-wide leaf).
// Returns true when ANY and a triangle was accepted.
template <bool ANY, bool COUNT, uint32_t ENDBIT = 1u>
__device__ __forceinline__ bool leaf_test(const TriRec* __restrict__ tris, uint32_t j, const Ray& r, Hit& h,
                                          uint32_t instIndex, uint64_t& nTris)
{
  while (true)
  {
    const float4* q = reinterpret_cast<const float4*>(tris + j);
    const float4 A = __ldg(q + 0);
    const float4 e1 = __ldg(q + 1);
    const float4 e2 = __ldg(q + 2);
    if (COUNT) nTris++;
    // pvec = cross(dir, e2), tvec = pos - A, qvec = cross(tvec, e1)
    const float px = __fsub_rn(__fmul_rn(r.dy, e2.z), __fmul_rn(r.dz, e2.y));
    const float py = __fsub_rn(__fmul_rn(r.dz, e2.x), __fmul_rn(r.dx, e2.z));
    const float pz = __fsub_rn(__fmul_rn(r.dx, e2.y), __fmul_rn(r.dy, e2.x));
    const float tx = __fsub_rn(r.ox, A.x);
    const float ty = __fsub_rn(r.oy, A.y);
    const float tz = __fsub_rn(r.oz, A.z);
    const float qx = __fsub_rn(__fmul_rn(ty, e1.z), __fmul_rn(tz, e1.y));
    const float qy = __fsub_rn(__fmul_rn(tz, e1.x), __fmul_rn(tx, e1.z));
    const float qz = __fsub_rn(__fmul_rn(tx, e1.y), __fmul_rn(ty, e1.x));
    const float det = __fadd_rn(__fadd_rn(__fmul_rn(e1.x, px), __fmul_rn(e1.y, py)), __fmul_rn(e1.z, pz));
    const float invDet = __frcp_rn(det);  // correctly rounded: the value of 1.0f / det
    const float v = __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(tx, px), __fmul_rn(ty, py)), __fmul_rn(tz, pz)), invDet);
    const float u = __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(qx, r.dx), __fmul_rn(qy, r.dy)), __fmul_rn(qz, r.dz)), invDet);
    const float t = __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(e2.x, qx), __fmul_rn(e2.y, qy)), __fmul_rn(e2.z, qz)), invDet);
    // 1.0f + 1e-6f rounds to 1 + 2^-20 in binary32
    if (v >= -1e-6f && u >= -1e-6f && __fadd_rn(u, v) <= 0x1.00001p+0f && t > r.tNear && t < h.t)
    {
      h.t = t;
      h.u = u;
      h.v = v;
      h.prim = j;
      h.inst = instIndex;
      if (ANY) return true;
    }
    if (__float_as_uint(A.w) & ENDBIT) return false;  // last triangle of the leaf
    j++;
  }
}

// ------------------------------------------------------- watertight triangle test
// Woop, Benthin & Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1),
// 2013: the ray's dominant axis becomes z (kx, ky keep the winding), the
// triangle is translated to the ray origin and sheared so that the ray runs
// along +z, and the signs of the three 2D edge functions at the origin decide
// the hit (both windings accepted).  The paper re-evaluates an edge function
// in double precision when it comes out zero; here each one is Kahan's
// difference of products (the rounding error of one product recovered by an
// FMA), whose relative error stays below 2 ulp, so its sign is exact in FP32
// and the test needs no FP64.  An edge shared by two triangles then gets
// exactly opposite signs on both sides: no ray passes between them.  Records
// hold the vertices {A, B, C} (w: flags, triangle id, 0).  Outputs match the
// Moller-Trumbore fields: u = the weight of C, v = the weight of B.
// a*b - c*d with the rounding error of c*d restored (Kahan).
__device__ __forceinline__ float diff_of_products(float a, float b, float c, float d)
{
  const float w = __fmul_rn(c, d);
  const float e = __fmaf_rn(-c, d, w);
  const float f = __fmaf_rn(a, b, -w);
  return __fadd_rn(f, e);
}

template <bool ANY, bool COUNT, uint32_t ENDBIT = 1u>
__device__ __forceinline__ bool leaf_test_wt(const TriRec* __restrict__ tris, uint32_t j, const Ray& r, Hit& h,
                                             uint32_t instIndex, uint64_t& nTris)
{
  const WtRay& w = r.w;
  while (true)
  {
    const float4* q = reinterpret_cast<const float4*>(tris + j);
    const float4 A = __ldg(q + 0);
    const float4 B = __ldg(q + 1);
    const float4 Cv = __ldg(q + 2);
    if (COUNT) nTris++;
    const float a0 = __fsub_rn(A.x, r.ox), a1 = __fsub_rn(A.y, r.oy), a2 = __fsub_rn(A.z, r.oz);
    const float b0 = __fsub_rn(B.x, r.ox), b1 = __fsub_rn(B.y, r.oy), b2 = __fsub_rn(B.z, r.oz);
    const float c0 = __fsub_rn(Cv.x, r.ox), c1 = __fsub_rn(Cv.y, r.oy), c2 = __fsub_rn(Cv.z, r.oz);
    const float az = pick3(a0, a1, a2, w.kz), bz = pick3(b0, b1, b2, w.kz), cz = pick3(c0, c1, c2, w.kz);
    const float ax = __fsub_rn(pick3(a0, a1, a2, w.kx), __fmul_rn(w.sx, az));
    const float ay = __fsub_rn(pick3(a0, a1, a2, w.ky), __fmul_rn(w.sy, az));
    const float bx = __fsub_rn(pick3(b0, b1, b2, w.kx), __fmul_rn(w.sx, bz));
    const float by = __fsub_rn(pick3(b0, b1, b2, w.ky), __fmul_rn(w.sy, bz));
    const float cx = __fsub_rn(pick3(c0, c1, c2, w.kx), __fmul_rn(w.sx, cz));
    const float cy = __fsub_rn(pick3(c0, c1, c2, w.ky), __fmul_rn(w.sy, cz));
    const float U = diff_of_products(cx, by, cy, bx);
    const float V = diff_of_products(ax, cy, ay, cx);
    const float W = diff_of_products(bx, ay, by, ax);
    const bool outside = (U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f);
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (!outside && det != 0.0f)
    {
      const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, __fmul_rn(w.sz, az)), __fmul_rn(V, __fmul_rn(w.sz, bz))),
                                __fmul_rn(W, __fmul_rn(w.sz, cz)));
      const float inv = __frcp_rn(det);
      const float t = __fmul_rn(T, inv);
      if (t > r.tNear && t < h.t)
      {
        h.t = t;
        h.u = __fmul_rn(W, inv);
        h.v = __fmul_rn(V, inv);
        h.prim = j;
        h.inst = instIndex;
        if (ANY) return true;
      }
    }
    if (__float_as_uint(A.w) & ENDBIT) return false;  // last triangle of the leaf
    j++;
  }
}

// The scene's triangle test: 0 Moller-Trumbore (the reference's), 1 watertight.
template <int TRI, bool ANY, bool COUNT, uint32_t ENDBIT>
__device__ __forceinline__ bool test_leaf(const TriRec* __restrict__ tris, uint32_t j, const Ray& r, Hit& h,
                                          uint32_t instIndex, uint64_t& nTris)
{
  if constexpr (TRI == 1) return leaf_test_wt<ANY, COUNT, ENDBIT>(tris, j, r, h, instIndex, nTris);
  else return leaf_test<ANY, COUNT, ENDBIT>(tris, j, r, h, instIndex, nTris);
}

// ---------------------------------------------------------------- 4-wide nodes
// Decoded child boxes of one 4-wide node.
struct Boxes4
{
  float lo[3][4], hi[3][4];
  uint4 ref;
};

__device__ __forceinline__ void load_node4(const Node4F32* __restrict__ n, Boxes4& B)
{
  const float4* p = reinterpret_cast<const float4*>(n);
  const float4 lx = __ldg(p + 0), ly = __ldg(p + 1), lz = __ldg(p + 2);
  const float4 hx = __ldg(p + 3), hy = __ldg(p + 4), hz = __ldg(p + 5);
  B.ref = __ldg(reinterpret_cast<const uint4*>(p + 6));
  B.lo[0][0] = lx.x; B.lo[0][1] = lx.y; B.lo[0][2] = lx.z; B.lo[0][3] = lx.w;
  B.lo[1][0] = ly.x; B.lo[1][1] = ly.y; B.lo[1][2] = ly.z; B.lo[1][3] = ly.w;
  B.lo[2][0] = lz.x; B.lo[2][1] = lz.y; B.lo[2][2] = lz.z; B.lo[2][3] = lz.w;
  B.hi[0][0] = hx.x; B.hi[0][1] = hx.y; B.hi[0][2] = hx.z; B.hi[0][3] = hx.w;
  B.hi[1][0] = hy.x; B.hi[1][1] = hy.y; B.hi[1][2] = hy.z; B.hi[1][3] = hy.w;
  B.hi[2][0] = hz.x; B.hi[2][1] = hz.y; B.hi[2][2] = hz.z; B.hi[2][3] = hz.w;
}

__device__ __forceinline__ float2 h2f(uint32_t w) { return __half22float2(*reinterpret_cast<const __half2*>(&w)); }

__device__ __forceinline__ void load_node4(const Node4F16* __restrict__ n, Boxes4& B)
{
  const uint4* p = reinterpret_cast<const uint4*>(n);
  const uint4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2);
  B.ref = __ldg(p + 3);
  const uint32_t aw[4] = {a.x, a.y, a.z, a.w}, bw[4] = {b.x, b.y, b.z, b.w}, cw[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
  for (int k = 0; k < 4; k++)
  {
    const float2 xy = h2f(aw[k]), zx = h2f(bw[k]), yz = h2f(cw[k]);
    B.lo[0][k] = xy.x; B.lo[1][k] = xy.y; B.lo[2][k] = zx.x;
    B.hi[0][k] = zx.y; B.hi[1][k] = yz.x; B.hi[2][k] = yz.y;
  }
}

__device__ __forceinline__ void load_node4(const Node4Q8* __restrict__ n, Boxes4& B)
{
  const uint4* p = reinterpret_cast<const uint4*>(n);
  const float4 f = __ldg(reinterpret_cast<const float4*>(p));
  const uint4 q0 = __ldg(p + 1), q1 = __ldg(p + 2);
  B.ref = __ldg(p + 3);
  const uint32_t e = __float_as_uint(f.w);
  const float org[3] = {f.x, f.y, f.z};
  const float sc[3] = {__int_as_float((int)(((e & 0xFFu) - 128u + 127u) << 23)),
                       __int_as_float((int)((((e >> 8) & 0xFFu) - 128u + 127u) << 23)),
                       __int_as_float((int)((((e >> 16) & 0xFFu) - 128u + 127u) << 23))};
  const uint32_t w[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
#pragma unroll
  for (int k = 0; k < 4; k++)
#pragma unroll
    for (int c = 0; c < 3; c++)
    {
      // origin + q * 2^e: the product is exact, so one fused add rounds like the encoder's add
      B.lo[c][k] = fmaf((float)((w[c] >> (8 * k)) & 0xFFu), sc[c], org[c]);
      B.hi[c][k] = fmaf((float)((w[3 + c] >> (8 * k)) & 0xFFu), sc[c], org[c]);
    }
}

template <int LAYOUT> struct Node4Type;
template <> struct Node4Type<1> { using type = Node4F32; };
template <> struct Node4Type<2> { using type = Node4F16; };
template <> struct Node4Type<3> { using type = Node4Q8; };

__device__ __forceinline__ void cswap(float& ka, uint32_t& va, float& kb, uint32_t& vb)
{
  const bool s = kb < ka;
  const float tk = s ? kb : ka;
  const uint32_t tv = s ? vb : va;
  kb = s ? ka : kb;
  vb = s ? va : vb;
  ka = tk;
  va = tv;
}

// Per-lane traversal state.
struct Lane
{
  Ray      r;
  Hit      h;
  float4   po, di;    // the ray as given (world space)
  uint32_t ray;       // ray index or kNoRay
  uint32_t inst;      // current instance
  uint32_t instEnd;   // one past the last instance this ray is traced against
  const void*   nodes;  // the current instance's records (binary) or 4-wide nodes
  const TriRec* tris;   // the current instance's triangle records
  uint32_t cur;       // current record / leaf reference
  int      top;       // stack depth
  int      base;      // stack depth at which the current instance's traversal began
  uint32_t tnext;     // next record of the current TLAS leaf run, or kNoRay
  uint32_t budget;    // steps left for this ray
};

// Upper bound on the steps of one ray: far above any real traversal (a ray
// visits each node at most once per instance); reaching it means a broken
// tree, and the ray ends as a miss with kErrStepBudget instead of looping.
constexpr uint32_t kStepBudget = 1u << 24;

// The first lane to run out of budget records its state after the error word:
// [1] = 1 (taken), [2] ray, [3] current ref, [4] stack depth.
template <typename LaneT>
__device__ __forceinline__ bool out_of_budget(LaneT& L, uint32_t* errorWord)
{
  if (L.budget-- != 0u) return false;
  atomicOr(errorWord, kErrStepBudget);
  if (atomicCAS(errorWord + 1, 0u, 1u) == 0u)
  {
    errorWord[2] = L.ray;
    errorWord[3] = L.cur;
    errorWord[4] = (uint32_t)L.top;
  }
  return true;
}

// Makes instance k the lane's current instance: its ray, and its node and
// triangle arrays held in registers for the steps that follow.
template <int LAYOUT>
__device__ __forceinline__ void enter_instance(Lane& L, const InstanceDesc* __restrict__ inst, uint32_t k)
{
  const InstanceDesc& d = inst[k];
  L.inst = k;
  make_ray(d, L.po, L.di, L.r);
  L.nodes = LAYOUT == 0 ? static_cast<const void*>(d.recs) : d.nodes4;
  L.tris = d.tris;
  L.cur = 0;  // record / node 0 = the root
}

// Advances the lane's instance cursor to the next instance with triangles,
// starting at `from` and ending before L.instEnd; prepares the ray for it.
// Returns false when none is left.
template <int LAYOUT>
__device__ __forceinline__ bool begin_instance(Lane& L, const InstanceDesc* __restrict__ inst, uint32_t from)
{
  for (uint32_t k = from; k < L.instEnd; k++)
    if (inst[k].valid)
    {
      enter_instance<LAYOUT>(L, inst, k);
      L.top = 0;
      L.base = 0;
      return true;
    }
  return false;
}

template <int LAYOUT> struct EndBit
{
  static constexpr uint32_t value = LAYOUT == 0 ? 1u : 2u;  // flag bit that ends a leaf of this layout
};

// Visits the internal node L.cur: tests its children, continues with the
// nearest hit child (child 0 on equal entry distance) and pushes the others,
// farthest first.  Returns 1 when no child is hit (the caller pops), 0
// otherwise, -1 when the stack bound would be exceeded (reported).
// One child pair of a binary tree: BVH2TraverseC32's decisions
// (core/BVH2CommonRT.cpp:88-113).
template <bool COUNT, int THREADS, int DEPTH, bool SPILL, typename LaneT>
__device__ __forceinline__ int visit_pair(LaneT& L, const PairRec* __restrict__ recs, Stack<THREADS, SPILL>& st,
                                          uint64_t& nPairs, uint32_t* errorWord)
{
  const float4* p = reinterpret_cast<const float4*>(recs + L.cur);
  const float4 a = __ldg(p + 0);
  const float4 b = __ldg(p + 1);
  const float4 c = __ldg(p + 2);
  const uint4 e = __ldg(reinterpret_cast<const uint4*>(p + 3));
  if (COUNT) nPairs++;
  float t0n, t0f, t1n, t1f;
  slab(L.r, a.x, a.y, a.z, a.w, b.x, b.y, t0n, t0f);
  slab(L.r, b.z, b.w, c.x, c.y, c.z, c.w, t1n, t1f);
  const bool h0 = (t0n <= t0f) && (t0f >= L.r.tNear) && (t0n <= L.h.t);
  const bool h1 = (t1n <= t1f) && (t1f >= L.r.tNear) && (t1n <= L.h.t);
  if (!h0 && !h1) return 1;
  L.cur = h0 ? e.x : e.y;
  if (h0 && h1)
  {
    const bool first0 = (t0n <= t1n);
    L.cur = first0 ? e.x : e.y;
    if (L.top >= DEPTH)
    {
      atomicOr(errorWord, kErrStack);
      return -1;
    }
    st.put(L.top, first0 ? e.y : e.x);
    L.top++;
  }
  return 0;
}

template <int LAYOUT, bool ANY, bool COUNT, int THREADS, int DEPTH, bool SPILL, typename LaneT>
__device__ __forceinline__ int visit_node(LaneT& L, Stack<THREADS, SPILL>& st, uint64_t& nPairs, uint32_t* errorWord)
{
  if constexpr (LAYOUT != 0)
  {
    // 4-wide node: HeavyRT's BVH4 order (core/BVH4CommonRT.cpp:49-246)
    using N = typename Node4Type<LAYOUT>::type;
    Boxes4 B;
    load_node4(reinterpret_cast<const N*>(L.nodes) + L.cur, B);
    if (COUNT) nPairs++;
    float key[4];
    uint32_t ref[4] = {B.ref.x, B.ref.y, B.ref.z, B.ref.w};
#pragma unroll
    for (int k = 0; k < 4; k++)
    {
      float tn, tf;
      slab(L.r, B.lo[0][k], B.lo[1][k], B.lo[2][k], B.hi[0][k], B.hi[1][k], B.hi[2][k], tn, tf);
      const bool hit = ref[k] != kEmptyRef && tn <= tf && tf >= L.r.tNear && tn <= L.h.t;
      key[k] = hit ? tn : INFINITY;
      ref[k] = hit ? ref[k] : kEmptyRef;
    }
    if constexpr (ANY)
    {
      // any hit: the answer does not depend on the visit order, so the hit
      // children are taken in slot order without sorting
      uint32_t first = kEmptyRef;
#pragma unroll
      for (int k = 3; k >= 0; k--)
      {
        if (ref[k] == kEmptyRef) continue;
        if (first != kEmptyRef)
        {
          if (L.top >= DEPTH)
          {
            atomicOr(errorWord, kErrStack);
            return -1;
          }
          st.put(L.top, first);
          L.top++;
        }
        first = ref[k];
      }
      if (first == kEmptyRef) return 1;
      L.cur = first;
      return 0;
    }
    cswap(key[0], ref[0], key[1], ref[1]);
    cswap(key[2], ref[2], key[3], ref[3]);
    cswap(key[0], ref[0], key[2], ref[2]);
    cswap(key[1], ref[1], key[3], ref[3]);
    cswap(key[1], ref[1], key[2], ref[2]);
    int f = 0;
    while (f < 4 && ref[f] == kEmptyRef) f++;
    if (f == 4) return 1;
    L.cur = ref[f];
#pragma unroll
    for (int k = 3; k >= 1; k--)
      if (k > f && ref[k] != kEmptyRef)
      {
        if (L.top >= DEPTH)
        {
          atomicOr(errorWord, kErrStack);
          return -1;
        }
        st.put(L.top, ref[k]);
        L.top++;
      }
    return 0;
  }
  else
    return visit_pair<COUNT, THREADS, DEPTH, SPILL>(L, reinterpret_cast<const PairRec*>(L.nodes), st, nPairs,
                                                    errorWord);
}

// One traversal step (an internal node, or a leaf followed by a pop).
// Returns true when the lane's ray is finished.
// Ray of the lane in world space (the instance tree is not transformed).
__device__ __forceinline__ void world_ray(Lane& L)
{
  L.r.tNear = L.po.w;
  L.r.ox = L.po.x; L.r.oy = L.po.y; L.r.oz = L.po.z;
  L.r.dx = L.di.x; L.r.dy = L.di.y; L.r.dz = L.di.z;
  L.r.ix = safe_inv(L.r.dx);
  L.r.iy = safe_inv(L.r.dy);
  L.r.iz = safe_inv(L.r.dz);
  wt_setup(L.r.dx, L.r.dy, L.r.dz, L.r.w);
}

__device__ __forceinline__ void tlas_begin(Lane& L)
{
  L.inst = kTlasMode;
  world_ray(L);
  L.cur = 0;
  L.top = 0;
  L.base = 0;
  L.tnext = kNoRay;
}

// Pops the instance tree's stack; true when the ray is finished.
template <int THREADS, bool SPILL>
__device__ __forceinline__ bool tlas_pop(Lane& L, const Stack<THREADS, SPILL>& st)
{
  if (L.top == 0) return true;
  L.top--;
  L.cur = st.get(L.top);
  return false;
}

// Enters the next instance (with triangles) of the current TLAS leaf run; when
// the run is done, returns to the instance tree.  True when the ray is finished.
template <int LAYOUT, int THREADS, bool SPILL>
__device__ __forceinline__ bool tlas_next(Lane& L, const InstanceDesc* __restrict__ inst, const Tlas& tl,
                                          const Stack<THREADS, SPILL>& st)
{
  while (L.tnext != kNoRay)
  {
    const float4* q = reinterpret_cast<const float4*>(tl.tris + L.tnext);
    const uint32_t flags = __float_as_uint(__ldg(q).w);
    const uint32_t k = __float_as_uint(__ldg(q + 1).w);
    L.tnext = (flags & 1u) ? kNoRay : L.tnext + 1;
    if (k < tl.nInst && inst[k].valid)
    {
      enter_instance<LAYOUT>(L, inst, k);
      L.base = L.top;
      return false;
    }
  }
  L.inst = kTlasMode;
  world_ray(L);
  return tlas_pop<THREADS, SPILL>(L, st);
}

template <int LAYOUT, int TRI, bool ANY, bool COUNT, int THREADS, bool TLAS, bool SPILL>
__device__ __forceinline__ bool step(Lane& L, const InstanceDesc* __restrict__ inst, const Tlas& tl,
                                     Stack<THREADS, SPILL>& st, uint64_t& nPairs, uint64_t& nTris, uint32_t* errorWord)
{
  constexpr int DEPTH = StackDepth<LAYOUT, TLAS>::value;
  if (TLAS && L.inst == kTlasMode)
  {
    // instance tree: a pair of instance boxes, or a leaf (a run of instances)
    if ((L.cur & kLeafBit) == 0u)
    {
      const int r = visit_pair<COUNT, THREADS, DEPTH, SPILL>(L, tl.recs, st, nPairs, errorWord);
      if (r < 0) return true;
      return r == 1 ? tlas_pop<THREADS, SPILL>(L, st) : false;
    }
    if (L.cur == kEmptyRef) return tlas_pop<THREADS, SPILL>(L, st);
    L.tnext = L.cur & ~kLeafBit;
    return tlas_next<LAYOUT, THREADS, SPILL>(L, inst, tl, st);
  }
  bool pop;
  if ((L.cur & kLeafBit) == 0u)
  {
    const int r = visit_node<LAYOUT, ANY, COUNT, THREADS, DEPTH, SPILL>(L, st, nPairs, errorWord);
    if (r < 0) return true;
    pop = (r == 1);
  }
  else
  {
    if (L.cur != kEmptyRef &&
        test_leaf<TRI, ANY, COUNT, EndBit<LAYOUT>::value>(L.tris, L.cur & ~kLeafBit, L.r, L.h, L.inst, nTris))
      return true;  // any-hit found
    pop = true;
  }
  if (pop)
  {
    if (L.top > L.base)
    {
      L.top--;
      L.cur = st.get(L.top);
      return false;
    }
    if (TLAS) return tlas_next<LAYOUT, THREADS, SPILL>(L, inst, tl, st);
    return !begin_instance<LAYOUT>(L, inst, L.inst + 1);
  }
  return false;
}

// The hit holds the instance's index; its instance and geometry ids are read
// once, here.
template <bool ANY>
__device__ __forceinline__ void write_result(const Lane& L, const InstanceDesc* __restrict__ inst, void* out)
{
  const bool hit = L.h.prim != 0xFFFFFFFFu;
  if (ANY)
    reinterpret_cast<uint8_t*>(out)[L.ray] = hit ? 1 : 0;
  else
  {
    const uint32_t instId = hit ? inst[L.h.inst].instId : 0xFFFFFFFFu;
    const uint32_t geomId = hit ? inst[L.h.inst].geomId : 0xFFFFFFFFu;
    store_record(reinterpret_cast<float4*>(reinterpret_cast<hrt_hit*>(out) + L.ray),
                 make_float4(L.h.t, __uint_as_float(L.h.prim), __uint_as_float(instId), __uint_as_float(geomId)),
                 make_float4(L.h.u, L.h.v, 0.0f, 0.0f));
  }
}

// Instances a ray is traced against: all of them, or - for a segmented query -
// the one instance of the ray's segment (rayOffsets[0..nSeg] ascending, ray i
// in segment k when rayOffsets[k] <= i < rayOffsets[k+1]); an instance id out
// of range leaves the ray a miss.
struct Segments
{
  const uint32_t* rayOffsets;  // nullptr: no segments
  const uint32_t* segInst;
  uint32_t        nSeg;
  uint32_t        nInst;
};

__device__ __forceinline__ uint32_t first_instance(Lane& L, uint32_t i, const Segments& sg)
{
  if (sg.rayOffsets == nullptr)
  {
    L.instEnd = sg.nInst;
    return 0;
  }
  uint32_t lo = 0, hi = sg.nSeg;
  while (hi - lo > 1)
  {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(sg.rayOffsets + mid) <= i) lo = mid;
    else hi = mid;
  }
  const uint32_t k = __ldg(sg.segInst + lo);
  L.instEnd = k < sg.nInst ? k + 1 : 0;
  return k;
}

__device__ __forceinline__ void start_ray(Lane& L, uint32_t i, const float4* __restrict__ rays)
{
  L.ray = i;
  load_record(rays + 2 * (size_t)i, L.po, L.di);
  L.h.t = L.di.w;
  L.h.u = L.h.v = 0.0f;
  L.h.prim = L.h.inst = 0xFFFFFFFFu;
  L.budget = kStepBudget;
}

template <bool COUNT>
__device__ __forceinline__ void flush_counters(uint64_t nPairs, uint64_t nTris, unsigned long long* counters)
{
  if (!COUNT) return;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    nPairs += __shfl_down_sync(0xFFFFFFFFu, nPairs, o);
    nTris += __shfl_down_sync(0xFFFFFFFFu, nTris, o);
  }
  if ((threadIdx.x & 31) == 0)
  {
    atomicAdd(&counters[0], (unsigned long long)nPairs);
    atomicAdd(&counters[1], (unsigned long long)nTris);
  }
}

// Persistent warp pool.  Lanes run `steps` traversal steps between refills; a
// warp refills when at least `refill` lanes are idle (or all are).
template <int LAYOUT, int TRI, bool ANY, bool COUNT, int THREADS, bool TLAS, bool SPILL>
__global__ void __launch_bounds__(THREADS) k_trace_pool(const float4* __restrict__ rays, uint32_t n,
                                                        const InstanceDesc* __restrict__ inst, Segments sg, Tlas tl,
                                                        void* out, unsigned long long* counters, uint32_t* errorWord,
                                                        unsigned int* rayCounter, int steps, int refill,
                                                        int stackShared, RayOrder order)
{
  extern __shared__ uint32_t s_stack[];  // stackShared * THREADS entries
  uint32_t spill[SPILL ? StackDepth<LAYOUT, TLAS>::value : 1];
  Stack<THREADS, SPILL> st{s_stack + threadIdx.x, spill, stackShared};
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t ltMask = (1u << lane) - 1u;
  uint64_t nPairs = 0, nTris = 0;
  Lane L;
  L.ray = kNoRay;
  bool exhausted = false;
  while (true)
  {
    const uint32_t idle = __ballot_sync(0xFFFFFFFFu, L.ray == kNoRay);
    if (exhausted && idle == 0xFFFFFFFFu) break;
    if (!exhausted && (__popc(idle) >= refill || idle == 0xFFFFFFFFu))
    {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(rayCounter, (unsigned int)__popc(idle));
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base + (uint32_t)__popc(idle) >= order.nWork) exhausted = true;
      if (L.ray == kNoRay)
      {
        const uint32_t w = base + __popc(idle & ltMask);
        const uint32_t i = w < order.nWork ? work_ray(order, w, n) : kNoRay;
        if (i != kNoRay)
        {
          start_ray(L, i, rays);
          bool live = true;
          if (TLAS) tlas_begin(L);
          else live = begin_instance<LAYOUT>(L, inst, first_instance(L, i, sg));
          if (!live)
          {
            write_result<ANY>(L, inst, out);
            L.ray = kNoRay;
          }
        }
      }
    }
    if (L.ray != kNoRay)
    {
      for (int s = 0; s < steps; s++)
      {
        if (out_of_budget(L, errorWord) ||
            step<LAYOUT, TRI, ANY, COUNT, THREADS, TLAS, SPILL>(L, inst, tl, st, nPairs, nTris, errorWord))
        {
          write_result<ANY>(L, inst, out);
          L.ray = kNoRay;
          break;
        }
      }
    }
  }
  flush_counters<COUNT>(nPairs, nTris, counters);
}

// One thread per ray.
template <int LAYOUT, int TRI, bool ANY, bool COUNT, int THREADS, bool TLAS, bool SPILL>
__global__ void __launch_bounds__(THREADS) k_trace_grid(const float4* __restrict__ rays, uint32_t n,
                                                        const InstanceDesc* __restrict__ inst, Segments sg, Tlas tl,
                                                        void* out, unsigned long long* counters, uint32_t* errorWord,
                                                        int stackShared, RayOrder order)
{
  extern __shared__ uint32_t s_stack[];  // stackShared * THREADS entries
  uint32_t spill[SPILL ? StackDepth<LAYOUT, TLAS>::value : 1];
  Stack<THREADS, SPILL> st{s_stack + threadIdx.x, spill, stackShared};
  uint64_t nPairs = 0, nTris = 0;
  const uint32_t w = blockIdx.x * THREADS + threadIdx.x;
  const uint32_t i = w < order.nWork ? work_ray(order, w, n) : kNoRay;
  if (i != kNoRay)
  {
    Lane L;
    start_ray(L, i, rays);
    bool live = true;
    if (TLAS) tlas_begin(L);
    else live = begin_instance<LAYOUT>(L, inst, first_instance(L, i, sg));
    if (live)
      while (!out_of_budget(L, errorWord) &&
             !step<LAYOUT, TRI, ANY, COUNT, THREADS, TLAS, SPILL>(L, inst, tl, st, nPairs, nTris, errorWord)) {}
    write_result<ANY>(L, inst, out);
  }
  flush_counters<COUNT>(nPairs, nTris, counters);
}

// ------------------------------------------------ one instance, no transform
// A scene of one geometry under the identity transform (no instance tree, no
// segments) needs none of the instance state: the ray is used as given, the
// node and triangle arrays are kernel parameters, and the ray leaves after its
// last pop.  The lane keeps less state, so the kernel holds fewer registers
// and more warps fit on an SM; each ray's decisions are those of the general
// kernel.
struct Lane1
{
  Ray           r;
  Hit           h;
  uint32_t      ray;     // ray index or kNoRay
  uint32_t      cur;     // current node / leaf reference
  int           top;     // stack depth
  uint32_t      budget;  // steps left for this ray
  const void*   nodes;   // the geometry's binary records or 4-wide nodes
  const TriRec* tris;
};

__device__ __forceinline__ void start_ray_one(Lane1& L, uint32_t i, const float4* __restrict__ rays)
{
  float4 po, di;
  load_record(rays + 2 * (size_t)i, po, di);
  L.ray = i;
  L.r.ox = po.x; L.r.oy = po.y; L.r.oz = po.z; L.r.tNear = po.w;
  L.r.dx = di.x; L.r.dy = di.y; L.r.dz = di.z;
  L.r.ix = safe_inv(di.x);
  L.r.iy = safe_inv(di.y);
  L.r.iz = safe_inv(di.z);
  wt_setup(di.x, di.y, di.z, L.r.w);
  L.h.t = di.w;
  L.h.u = L.h.v = 0.0f;
  L.h.prim = L.h.inst = 0xFFFFFFFFu;
  L.cur = 0;
  L.top = 0;
  L.budget = kStepBudget;
}

// One step of the single-instance kernel; true when the ray is finished.
template <int LAYOUT, int TRI, bool ANY, int THREADS, bool SPILL>
__device__ __forceinline__ bool step_one(Lane1& L, Stack<THREADS, SPILL>& st, uint32_t* errorWord)
{
  constexpr int DEPTH = StackDepth<LAYOUT, false>::value;
  uint64_t none = 0;
  if ((L.cur & kLeafBit) == 0u)
  {
    const int r = visit_node<LAYOUT, ANY, false, THREADS, DEPTH, SPILL>(L, st, none, errorWord);
    if (r < 0) return true;
    if (r == 0) return false;
  }
  else if (L.cur != kEmptyRef &&
           test_leaf<TRI, ANY, false, EndBit<LAYOUT>::value>(L.tris, L.cur & ~kLeafBit, L.r, L.h, 0u, none))
    return true;  // any-hit found
  if (L.top == 0) return true;
  L.top--;
  L.cur = st.get(L.top);
  return false;
}

template <bool ANY>
__device__ __forceinline__ void write_result_one(const Lane1& L, uint32_t instId, uint32_t geomId, void* out)
{
  const bool hit = L.h.prim != 0xFFFFFFFFu;
  if (ANY)
    reinterpret_cast<uint8_t*>(out)[L.ray] = hit ? 1 : 0;
  else
  {
    store_record(reinterpret_cast<float4*>(reinterpret_cast<hrt_hit*>(out) + L.ray),
                 make_float4(L.h.t, __uint_as_float(L.h.prim), __uint_as_float(hit ? instId : 0xFFFFFFFFu),
                             __uint_as_float(hit ? geomId : 0xFFFFFFFFu)),
                 make_float4(L.h.u, L.h.v, 0.0f, 0.0f));
  }
}

// Persistent warp pool over one instance (the refill rule of k_trace_pool).
template <int LAYOUT, int TRI, bool ANY, int THREADS, bool SPILL>
__global__ void __launch_bounds__(THREADS) k_trace_one(const float4* __restrict__ rays, uint32_t n,
                                                       const void* __restrict__ nodes, const TriRec* __restrict__ tris,
                                                       uint32_t instId, uint32_t geomId, void* out,
                                                       uint32_t* errorWord, unsigned int* rayCounter, int steps,
                                                       int refill, int stackShared, RayOrder order)
{
  extern __shared__ uint32_t s_stack[];  // stackShared * THREADS entries
  uint32_t spill[SPILL ? StackDepth<LAYOUT, false>::value : 1];
  Stack<THREADS, SPILL> st{s_stack + threadIdx.x, spill, stackShared};
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t ltMask = (1u << lane) - 1u;
  Lane1 L;
  L.ray = kNoRay;
  L.nodes = nodes;
  L.tris = tris;
  bool exhausted = false;
  while (true)
  {
    const uint32_t idle = __ballot_sync(0xFFFFFFFFu, L.ray == kNoRay);
    if (exhausted && idle == 0xFFFFFFFFu) break;
    if (!exhausted && (__popc(idle) >= refill || idle == 0xFFFFFFFFu))
    {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(rayCounter, (unsigned int)__popc(idle));
      base = __shfl_sync(0xFFFFFFFFu, base, 0);
      if (base + (uint32_t)__popc(idle) >= order.nWork) exhausted = true;
      if (L.ray == kNoRay)
      {
        const uint32_t w = base + __popc(idle & ltMask);
        const uint32_t i = w < order.nWork ? work_ray(order, w, n) : kNoRay;
        if (i != kNoRay) start_ray_one(L, i, rays);
      }
    }
    if (L.ray != kNoRay)
    {
      for (int s = 0; s < steps; s++)
      {
        if (out_of_budget(L, errorWord) || step_one<LAYOUT, TRI, ANY, THREADS, SPILL>(L, st, errorWord))
        {
          write_result_one<ANY>(L, instId, geomId, out);
          L.ray = kNoRay;
          break;
        }
      }
    }
  }
}

// One thread per ray over one instance: a warp's 32 consecutive rays end
// together, so their results go out as one contiguous kilobyte (results
// written in place over the host link want this).
template <int LAYOUT, int TRI, bool ANY, int THREADS, bool SPILL>
__global__ void __launch_bounds__(THREADS)
    k_trace_one_grid(const float4* __restrict__ rays, uint32_t n, const void* __restrict__ nodes,
                     const TriRec* __restrict__ tris, uint32_t instId, uint32_t geomId, void* out, uint32_t* errorWord,
                     int stackShared, RayOrder order)
{
  extern __shared__ uint32_t s_stack[];  // stackShared * THREADS entries
  uint32_t spill[SPILL ? StackDepth<LAYOUT, false>::value : 1];
  Stack<THREADS, SPILL> st{s_stack + threadIdx.x, spill, stackShared};
  const uint32_t w = blockIdx.x * THREADS + threadIdx.x;
  const uint32_t i = w < order.nWork ? work_ray(order, w, n) : kNoRay;
  if (i == kNoRay) return;
  Lane1 L;
  L.nodes = nodes;
  L.tris = tris;
  start_ray_one(L, i, rays);
  while (!out_of_budget(L, errorWord) && !step_one<LAYOUT, TRI, ANY, THREADS, SPILL>(L, st, errorWord)) {}
  write_result_one<ANY>(L, instId, geomId, out);
}

// Dynamic shared memory of a traversal kernel: `shared` stack entries per
// thread; above 48 KB a block needs the opt-in attribute.
template <typename K> cudaError_t allow_smem(K kernel, size_t smem)
{
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <int LAYOUT, int TRI, bool ANY, int THREADS, bool SPILL>
cudaError_t launch_one(const TraceArgs& a, const TraceConfig& c, int numSMs, cudaStream_t s)
{
  const uint32_t n = (uint32_t)a.n;
  const int shared = shared_entries<StackDepth<LAYOUT, false>::value>(c.stackEntries);
  const size_t smem = sizeof(uint32_t) * (size_t)shared * THREADS;
  const RayOrder order = ray_order(n, c.imageWidth);
  const InstanceDesc& d = *a.one;
  const void* nodes = LAYOUT == 0 ? static_cast<const void*>(d.recs) : d.nodes4;
  // launch configuration, with the L2 access-policy window when one is asked for
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t lc = {};
  lc.blockDim = dim3(THREADS);
  lc.dynamicSmemBytes = smem;
  lc.stream = s;
  if (a.persistBytes)
  {
    attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[0].val.accessPolicyWindow.base_ptr = const_cast<void*>(a.persistBase);
    attr[0].val.accessPolicyWindow.num_bytes = a.persistBytes;
    attr[0].val.accessPolicyWindow.hitRatio = a.persistHitRatio;
    attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    lc.attrs = attr;
    lc.numAttrs = 1;
  }
  if (!c.persistent)
  {
    cudaError_t e = allow_smem(k_trace_one_grid<LAYOUT, TRI, ANY, THREADS, SPILL>, smem);
    if (e != cudaSuccess) return e;
    lc.gridDim = dim3((uint32_t)(((uint64_t)order.nWork + THREADS - 1) / THREADS));
    return cudaLaunchKernelEx(&lc, k_trace_one_grid<LAYOUT, TRI, ANY, THREADS, SPILL>, a.rays, n, nodes, d.tris,
                              d.instId, d.geomId, a.hits, a.errorWord, shared, order);
  }
  cudaError_t e = allow_smem(k_trace_one<LAYOUT, TRI, ANY, THREADS, SPILL>, smem);
  if (e != cudaSuccess) return e;
  int perSM = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_trace_one<LAYOUT, TRI, ANY, THREADS, SPILL>, THREADS,
                                                    smem);
  if (e != cudaSuccess) return e;
  if (perSM < 1) perSM = 1;
  uint64_t blocks = (uint64_t)numSMs * perSM;
  const uint64_t need = ((uint64_t)order.nWork + THREADS - 1) / THREADS;
  if (blocks > need) blocks = need;
  e = cudaMemsetAsync(a.rayCounter, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  lc.gridDim = dim3((uint32_t)blocks);
  return cudaLaunchKernelEx(&lc, k_trace_one<LAYOUT, TRI, ANY, THREADS, SPILL>, a.rays, n, nodes, d.tris, d.instId,
                            d.geomId, a.hits, a.errorWord, a.rayCounter, c.stepsPerRefill, c.refillLanes, shared,
                            order);
}

// The short-stack variant only when the requested size leaves part of the
// depth bound to local memory.
template <int LAYOUT, int TRI, bool ANY, int THREADS>
cudaError_t launch_one_any_stack(const TraceArgs& a, const TraceConfig& c, int numSMs, cudaStream_t s)
{
  constexpr int DEPTH = StackDepth<LAYOUT, false>::value;
  return shared_entries<DEPTH>(c.stackEntries) < DEPTH ? launch_one<LAYOUT, TRI, ANY, THREADS, true>(a, c, numSMs, s)
                                                       : launch_one<LAYOUT, TRI, ANY, THREADS, false>(a, c, numSMs, s);
}

template <int LAYOUT, int TRI>
cudaError_t trace_one(const TraceArgs& a, int kind, const TraceConfig& c, int numSMs, cudaStream_t s)
{
  switch (c.threadsPerBlock)
  {
    case 64:
      return kind == 0 ? launch_one_any_stack<LAYOUT, TRI, false, 64>(a, c, numSMs, s)
                       : launch_one_any_stack<LAYOUT, TRI, true, 64>(a, c, numSMs, s);
    case 256:
      return kind == 0 ? launch_one_any_stack<LAYOUT, TRI, false, 256>(a, c, numSMs, s)
                       : launch_one_any_stack<LAYOUT, TRI, true, 256>(a, c, numSMs, s);
    default:
      return kind == 0 ? launch_one_any_stack<LAYOUT, TRI, false, 128>(a, c, numSMs, s)
                       : launch_one_any_stack<LAYOUT, TRI, true, 128>(a, c, numSMs, s);
  }
}

template <int LAYOUT, int TRI, bool ANY, bool COUNT, int THREADS, bool TLAS, bool SPILL>
cudaError_t launch(const TraceArgs& a, const TraceConfig& c, int numSMs, cudaStream_t s)
{
  const uint32_t n = (uint32_t)a.n;
  const Segments sg{a.rayOffsets, a.segInst, a.nSeg, a.nInst};
  const Tlas tl{a.tlasRecs, a.tlasTris, a.nInst};
  const int shared = SPILL ? shared_entries<StackDepth<LAYOUT, TLAS>::value>(c.stackEntries)
                           : StackDepth<LAYOUT, TLAS>::value;
  const size_t smem = sizeof(uint32_t) * (size_t)shared * THREADS;
  const RayOrder order = ray_order(n, c.imageWidth);
  if (c.persistent && !COUNT)
  {
    cudaError_t e = allow_smem(k_trace_pool<LAYOUT, TRI, ANY, COUNT, THREADS, TLAS, SPILL>, smem);
    if (e != cudaSuccess) return e;
    int perSM = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &perSM, k_trace_pool<LAYOUT, TRI, ANY, COUNT, THREADS, TLAS, SPILL>, THREADS, smem);
    if (e != cudaSuccess) return e;
    if (perSM < 1) perSM = 1;
    uint64_t blocks = (uint64_t)numSMs * perSM;
    const uint64_t need = ((uint64_t)order.nWork + THREADS - 1) / THREADS;
    if (blocks > need) blocks = need;
    e = cudaMemsetAsync(a.rayCounter, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
    k_trace_pool<LAYOUT, TRI, ANY, COUNT, THREADS, TLAS, SPILL><<<(uint32_t)blocks, THREADS, smem, s>>>(
        a.rays, n, a.inst, sg, tl, a.hits, a.counters, a.errorWord, a.rayCounter, c.stepsPerRefill, c.refillLanes,
        shared, order);
  }
  else
  {
    cudaError_t e = allow_smem(k_trace_grid<LAYOUT, TRI, ANY, COUNT, THREADS, TLAS, SPILL>, smem);
    if (e != cudaSuccess) return e;
    const uint64_t blocks = ((uint64_t)order.nWork + THREADS - 1) / THREADS;
    k_trace_grid<LAYOUT, TRI, ANY, COUNT, THREADS, TLAS, SPILL><<<(uint32_t)blocks, THREADS, smem, s>>>(
        a.rays, n, a.inst, sg, tl, a.hits, a.counters, a.errorWord, shared, order);
  }
  return cudaGetLastError();
}

template <int LAYOUT, int TRI, bool ANY, int THREADS, bool TLAS>
cudaError_t launch_any_stack(const TraceArgs& a, const TraceConfig& c, int numSMs, cudaStream_t s)
{
  constexpr int DEPTH = StackDepth<LAYOUT, TLAS>::value;
  return shared_entries<DEPTH>(c.stackEntries) < DEPTH
             ? launch<LAYOUT, TRI, ANY, false, THREADS, TLAS, true>(a, c, numSMs, s)
             : launch<LAYOUT, TRI, ANY, false, THREADS, TLAS, false>(a, c, numSMs, s);
}

template <int LAYOUT, int TRI, bool TLAS>
cudaError_t trace_tlas(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s)
{
  // counting runs: the whole stack in shared memory (the counts do not depend on it)
  if (counting)
    return kind == 0 ? launch<LAYOUT, TRI, false, true, 128, TLAS, false>(a, c, numSMs, s)
                     : launch<LAYOUT, TRI, true, true, 128, TLAS, false>(a, c, numSMs, s);
  switch (c.threadsPerBlock)
  {
    case 64:
      return kind == 0 ? launch_any_stack<LAYOUT, TRI, false, 64, TLAS>(a, c, numSMs, s)
                       : launch_any_stack<LAYOUT, TRI, true, 64, TLAS>(a, c, numSMs, s);
    case 256:
      return kind == 0 ? launch_any_stack<LAYOUT, TRI, false, 256, TLAS>(a, c, numSMs, s)
                       : launch_any_stack<LAYOUT, TRI, true, 256, TLAS>(a, c, numSMs, s);
    default:
      return kind == 0 ? launch_any_stack<LAYOUT, TRI, false, 128, TLAS>(a, c, numSMs, s)
                       : launch_any_stack<LAYOUT, TRI, true, 128, TLAS>(a, c, numSMs, s);
  }
}

// Counting runs use the one-thread-per-ray grid at 128 threads: the counts do
// not depend on the schedule.  A scene with an instance tree uses the
// two-level kernels, except in segmented queries (one instance per ray).  A
// scene of one untransformed instance uses the single-instance kernels.
template <int LAYOUT, int TRI>
cudaError_t trace_layout(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s)
{
  if (a.one != nullptr && !counting && a.rayOffsets == nullptr && a.tlasRecs == nullptr)
    return trace_one<LAYOUT, TRI>(a, kind, c, numSMs, s);
  if (a.tlasRecs != nullptr && a.rayOffsets == nullptr)
    return trace_tlas<LAYOUT, TRI, true>(a, kind, counting, c, numSMs, s);
  return trace_tlas<LAYOUT, TRI, false>(a, kind, counting, c, numSMs, s);
}

}  // namespace

// Per-layout entry points, one translation unit each (trace_l*.cu).
cudaError_t trace_l0(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_l1(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_l2(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_l3(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
// The same with the watertight triangle test (trace_w*.cu).
cudaError_t trace_w0(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_w1(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_w2(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);
cudaError_t trace_w3(const TraceArgs& a, int kind, int counting, const TraceConfig& c, int numSMs, cudaStream_t s);

}  // namespace hrt
