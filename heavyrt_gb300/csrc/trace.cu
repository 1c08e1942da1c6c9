// Nearest-hit / any-hit traversal of the LBVH.
//
// Each thread traces one ray through every instance: the decisions are those
// of HeavyRT's BVH2TraverseC32 (core/BVH2CommonRT.cpp:49-141) on the same
// binary tree - load the two children of the current node, slab-test both
// (core/raytrace_common.h:67-80), descend into the nearer hit child (child 0
// on equal entry distance), push the other, pop when neither is hit - and the
// leaf test is the reference's Moller-Trumbore with 1e-6 barycentric slack
// (core/BVH2CommonRT.cpp:9-47).  All float operations are explicit
// round-to-nearest intrinsics in the reference's evaluation order, so the
// results match the CPU reference bit for bit.
//
// Memory: a child pair is one 64-byte record (four 128-bit read-only loads), a
// triangle one 48-byte record (three); the short stack lives in shared memory,
// STACK entries per thread, interleaved by thread so that pushes and pops of a
// warp hit 32 different banks.
#include "hrt_kernels.cuh"
#include "../../include/hrt.h"

namespace hrt
{
namespace
{

constexpr int kThreads = 128;
constexpr int kStack   = 32;  // LBVH depth <= 30 for 30-bit codes: one push per level at most

struct Ray
{
  float ox, oy, oz, tNear;
  float dx, dy, dz;
  float ix, iy, iz;
};

// SafeInverse, core/raytrace_common.h:57-65.
__device__ __forceinline__ float safe_inv(float d)
{
  const float ooeps = 1.0e-36f;
  return __fdiv_rn(1.0f, fabsf(d) > ooeps ? d : copysignf(ooeps, d));
}

// RayBoxIntersection2, core/raytrace_common.h:67-80.
__device__ __forceinline__ void slab(const Ray& r, float bx0, float by0, float bz0, float bx1, float by1, float bz1,
                                     float& tn, float& tf)
{
  const float lo = __fmul_rn(r.ix, __fsub_rn(bx0, r.ox));
  const float hi = __fmul_rn(r.ix, __fsub_rn(bx1, r.ox));
  const float lo1 = __fmul_rn(r.iy, __fsub_rn(by0, r.oy));
  const float hi1 = __fmul_rn(r.iy, __fsub_rn(by1, r.oy));
  const float lo2 = __fmul_rn(r.iz, __fsub_rn(bz0, r.oz));
  const float hi2 = __fmul_rn(r.iz, __fsub_rn(bz1, r.oz));
  const float tmin = std_max(std_min(lo, hi), std_min(lo1, hi1));
  const float tmax = std_min(std_max(lo, hi), std_max(lo1, hi1));
  tn = std_max(tmin, std_min(lo2, hi2));
  tf = std_min(tmax, std_max(lo2, hi2));
}

struct Hit
{
  float    t, u, v;
  uint32_t prim, inst, geom;
};

// matmul4x3 / matmul3x3 (core/raytrace_common.h:82-90) with the column sum
// order ((m0*x + m1*y) + m2*z) + m3*w.
__device__ __forceinline__ float row_dot(const float* m, float x, float y, float z, float w)
{
  return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], x), __fmul_rn(m[1], y)), __fmul_rn(m[2], z)), __fmul_rn(m[3], w));
}

template <bool ANY, bool COUNT>
__device__ __forceinline__ bool traverse(const PairRec* __restrict__ recs, const TriRec* __restrict__ tris, const Ray& r,
                                         Hit& h, uint32_t instId, uint32_t geomId, uint32_t* __restrict__ stack,
                                         uint64_t& nPairs, uint64_t& nTris, uint32_t* errorWord)
{
  int top = 0;
  uint32_t cur = 0;  // record 0 = the root's two children
  while (top >= 0)
  {
    bool pop = false;
    if ((cur & kLeafBit) == 0u)
    {
      const float4* p = reinterpret_cast<const float4*>(recs + cur);
      const float4 a = __ldg(p + 0);
      const float4 b = __ldg(p + 1);
      const float4 c = __ldg(p + 2);
      const uint4 d = __ldg(reinterpret_cast<const uint4*>(p + 3));
      if (COUNT) nPairs++;
      float t0n, t0f, t1n, t1f;
      slab(r, a.x, a.y, a.z, a.w, b.x, b.y, t0n, t0f);
      slab(r, b.z, b.w, c.x, c.y, c.z, c.w, t1n, t1f);
      const bool h0 = (t0n <= t0f) && (t0f >= r.tNear) && (t0n <= h.t);
      const bool h1 = (t1n <= t1f) && (t1f >= r.tNear) && (t1n <= h.t);
      pop = !h0 && !h1;
      cur = h0 ? d.x : d.y;
      if (h0 && h1)
      {
        const bool first0 = (t0n <= t1n);
        cur = first0 ? d.x : d.y;
        if (top >= kStack)
        {
          atomicOr(errorWord, kErrStack);
          return false;
        }
        stack[top * kThreads] = first0 ? d.y : d.x;
        top++;
      }
    }
    else
    {
      if (cur != kEmptyRef)
      {
        uint32_t j = cur & ~kLeafBit;
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
          const float invDet = __fdiv_rn(1.0f, det);
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
            h.inst = instId;
            h.geom = geomId;
            if (ANY) return true;
          }
          if (__float_as_uint(A.w) & 1u) break;  // last triangle of the leaf
          j++;
        }
      }
      pop = true;
    }
    if (pop)
    {
      top--;
      cur = stack[(top > 0 ? top : 0) * kThreads];
    }
  }
  return false;
}

template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kThreads) k_trace(const float4* __restrict__ rays, uint64_t n,
                                                    const InstanceDesc* __restrict__ inst, uint32_t nInst, void* out,
                                                    unsigned long long* counters, uint32_t* errorWord)
{
  __shared__ uint32_t s_stack[kStack * kThreads];
  uint32_t* stack = s_stack + threadIdx.x;
  stack[0] = 0u;
  uint64_t nPairs = 0, nTris = 0;
  const uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i < n)
  {
    const float4 po = __ldg(rays + 2 * i + 0);
    const float4 di = __ldg(rays + 2 * i + 1);
    Hit h;
    h.t = di.w;
    h.u = h.v = 0.0f;
    h.prim = h.inst = h.geom = 0xFFFFFFFFu;
    bool any = false;
    for (uint32_t k = 0; k < nInst && !any; k++)
    {
      const InstanceDesc& d = inst[k];
      if (!d.valid) continue;
      Ray r;
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
      any = traverse<ANY, COUNT>(d.recs, d.tris, r, h, d.instId, d.geomId, stack, nPairs, nTris, errorWord);
    }
    if (ANY)
      reinterpret_cast<uint8_t*>(out)[i] = any ? 1 : 0;
    else
    {
      float4* o = reinterpret_cast<float4*>(reinterpret_cast<hrt_hit*>(out) + i);
      o[0] = make_float4(h.t, __uint_as_float(h.prim), __uint_as_float(h.inst), __uint_as_float(h.geom));
      o[1] = make_float4(h.u, h.v, 0.0f, 0.0f);
    }
  }
  if (COUNT)
  {
    // warp-aggregate, one atomic per warp and counter
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
}

}  // namespace

cudaError_t trace(const TraceArgs& a, int kind, int counting, int numSMs, cudaStream_t s)
{
  (void)numSMs;
  if (a.n == 0) return cudaSuccess;
  const uint64_t blocks = (a.n + kThreads - 1) / kThreads;
  if (blocks > 0x7FFFFFFFull) return cudaErrorInvalidValue;
  const dim3 g((uint32_t)blocks);
  if (kind == 0)
  {
    if (counting) k_trace<false, true><<<g, kThreads, 0, s>>>(a.rays, a.n, a.inst, a.nInst, a.hits, a.counters, a.errorWord);
    else k_trace<false, false><<<g, kThreads, 0, s>>>(a.rays, a.n, a.inst, a.nInst, a.hits, a.counters, a.errorWord);
  }
  else
  {
    if (counting) k_trace<true, true><<<g, kThreads, 0, s>>>(a.rays, a.n, a.inst, a.nInst, a.hits, a.counters, a.errorWord);
    else k_trace<true, false><<<g, kThreads, 0, s>>>(a.rays, a.n, a.inst, a.nInst, a.hits, a.counters, a.errorWord);
  }
  return cudaGetLastError();
}

}  // namespace hrt
