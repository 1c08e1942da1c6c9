// Whole frames of HeavyRT's two example renderers on the device: the rays are
// generated, traced through the scene and shaded without crossing the host
// link, with every value equal bit for bit to the renderers' own kernels.
//
//  * Eye-ray frame, EyeRayCaster (examples/01_eye_rays/eye_ray.cpp:10-74):
//    one ray per pixel (kernel_InitEyeRay, tNear 0, tFar MAXFLOAT), nearest
//    hit, colour 0 on a miss, else palette[primId % 20] (kernel_RayTrace).
//  * RTAO frame (examples/02_rtao/rtao.cpp:46-185): eye rays from the zNear /
//    zFar range, nearest hit, kernel_TraceEyeRay2's hit point and packed
//    shading normal, kernel_InitAORay's raysPerPixel cosine-distributed rays
//    from the renderer's 128x128 quasi-random sample tile
//    (rtao_host.cpp:383-414), any-hit (the renderer's closest-hit query with a
//    zero attenuation counts the same unoccluded samples), kernel_AO2Color.
//
// Rays are traced in EyeRayCaster's packed order (4x4 pixel blocks inside
// 2x2 super-blocks, kernel_PackXY) when both image sides are multiples of 8,
// row by row otherwise; the images do not depend on the order.  AO rays are
// compacted to the pixels with a hit, raysPerPixel consecutive rays each, in
// trace order; the frame synchronises its stream once to size that launch.
//
// Arithmetic: explicit round-to-nearest float operations in the reference's
// evaluation order (LiteMath as the checker's stand-in evaluates it).  The
// renderer's sin, cos and pow of a sample (MapSampleToCosineDistribution,
// examples/render_common.h:56-94) depend only on the tile entry; they are
// evaluated once per entry on the host, in double as the renderer does, and
// kept as a table on the device.  CoordinateSystem's second branch divides in
// double (render_common.h:49), done here with IEEE double operations.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "hrt_internal.cuh"
#include "raygen_common.cuh"

using namespace hrt;
using namespace hrt::api;
using hrt::rg::Mat4;

namespace
{

constexpr int      kThreads = 256;
constexpr int      kChunk = 4;  // items per thread in the compaction blocks
constexpr uint32_t kAoTile = HRT_AO_TILE_SIZE;
constexpr float    kHitBack = 10000000.0f;  // RTAO::AO_HIT_BACK

// EyeRayCaster's palette (examples/01_eye_rays/eye_ray.h:105-113).
__constant__ uint32_t c_palette[20] = {0xffe6194bu, 0xff3cb44bu, 0xffffe119u, 0xff0082c8u, 0xfff58231u,
                                       0xff911eb4u, 0xff46f0f0u, 0xfff032e6u, 0xffd2f53cu, 0xfffabebeu,
                                       0xff008080u, 0xffe6beffu, 0xffaa6e28u, 0xfffffac8u, 0xff800000u,
                                       0xffaaffc3u, 0xff808000u, 0xffffd8b1u, 0xff000080u, 0xff808080u};

// Pixel of the k-th traced ray.  Packed order = the inverse of
// SuperBlockIndex2DOpt (examples/01_eye_rays/eye_ray.cpp:106-127).
__device__ __forceinline__ void traced_pixel(uint64_t k, uint32_t width, int packed, uint32_t& x, uint32_t& y)
{
  if (!packed)
  {
    y = (uint32_t)(k / width);
    x = (uint32_t)(k % width);
    return;
  }
  const uint32_t superBlocksX = width >> 3;
  const uint32_t sb = (uint32_t)(k >> 6), quad = (uint32_t)(k >> 4) & 3u, local = (uint32_t)k & 15u;
  x = ((sb % superBlocksX) * 2u + (quad & 1u)) * 4u + (local & 3u);
  y = ((sb / superBlocksX) * 2u + (quad >> 1)) * 4u + (local >> 2);
}

__global__ void __launch_bounds__(kThreads) k_frame_eye_rays(Mat4 projInv, Mat4 worldViewInv, uint32_t width,
                                                             uint32_t height, int packed, float tNear, float tFar,
                                                             float4* __restrict__ rays, uint32_t* __restrict__ pixel)
{
  const uint64_t n = (uint64_t)width * height;
  for (uint64_t k = (uint64_t)blockIdx.x * kThreads + threadIdx.x; k < n; k += (uint64_t)gridDim.x * kThreads)
  {
    uint32_t x, y;
    traced_pixel(k, width, packed, x, y);
    float4 o, d;
    hrt::rg::eye_ray(projInv, worldViewInv, x, y, width, height, tNear, tFar, o, d);
    rays[2 * k + 0] = o;
    rays[2 * k + 1] = d;
    pixel[k] = y * width + x;
  }
}

// kernel_RayTrace's colour (examples/01_eye_rays/eye_ray.cpp:49-74).
__global__ void __launch_bounds__(kThreads) k_eye_colors(const hrt_hit* __restrict__ hits,
                                                         const uint32_t* __restrict__ pixel, uint64_t n,
                                                         uint32_t* __restrict__ colors)
{
  for (uint64_t k = (uint64_t)blockIdx.x * kThreads + threadIdx.x; k < n; k += (uint64_t)gridDim.x * kThreads)
  {
    const uint32_t prim = hits[k].primId;
    colors[pixel[k]] = prim == 0xFFFFFFFFu ? 0u : c_palette[prim % 20u];
  }
}

struct FrameGeom
{
  const float4*   verts;
  const uint32_t* sortedIdx;
  const float4*   normals;
  uint32_t        nTris;
};

// C++ float -> int conversion (truncation); NaN, undefined in C++, gives 0.
__device__ __forceinline__ int f2i(float f) { return f != f ? 0 : __float2int_rz(f); }

// encodeNormal (examples/render_common.h:114-124)
__device__ __forceinline__ uint32_t encode_normal(float nx, float ny, float nz)
{
  const int x = f2i(__fmul_rn(nx, 32767.0f));
  const int y = f2i(__fmul_rn(ny, 32767.0f));
  const uint32_t sign = (nz >= 0.0f) ? 0u : 1u;
  return ((uint32_t)(x & 0xfffe) | sign) | ((uint32_t)(y & 0xffff) << 16);
}

// mymul3x3 (examples/render_common.h:14-17): the whole column sum, w = 0.
__device__ __forceinline__ void mul3x3(const float* m, const float v[3], float o[3])
{
#pragma unroll
  for (int r = 0; r < 3; r++)
    o[r] = __fadd_rn(
        __fadd_rn(__fadd_rn(__fmul_rn(m[r], v[0]), __fmul_rn(m[4 + r], v[1])), __fmul_rn(m[8 + r], v[2])),
        __fmul_rn(m[12 + r], 0.0f));
}

// kernel_TraceEyeRay2 after the query (examples/02_rtao/rtao.cpp:81-131): one
// traced eye ray -> its pixel's hit point and packed shading normal, and the
// ray's flag (1 = the pixel gets AO rays).  The triangle is read from the
// geometry's index buffer in sorted order at the hit's primId (its sorted
// position), i.e. the triangle that was hit.
__global__ void __launch_bounds__(kThreads)
    k_rtao_positions(const float4* __restrict__ rays, const hrt_hit* __restrict__ hits,
                     const uint32_t* __restrict__ pixel, uint64_t n, const FrameGeom* __restrict__ geoms,
                     uint32_t nGeoms, const float* __restrict__ normMatrices, uint32_t nInst,
                     float4* __restrict__ positions, uint8_t* __restrict__ flag, uint32_t* errorWord)
{
  for (uint64_t k = (uint64_t)blockIdx.x * kThreads + threadIdx.x; k < n; k += (uint64_t)gridDim.x * kThreads)
  {
    const hrt_hit h = hits[k];
    float4 out;
    if (h.geomId == 0xFFFFFFFFu)
      out = make_float4(0.0f, kHitBack, 0.0f, __uint_as_float(encode_normal(0.0f, 1.0f, 0.0f)));
    else if (h.geomId >= nGeoms || h.instId >= nInst || h.primId >= geoms[h.geomId].nTris)
    {
      atomicOr(errorWord, kErrIndexRange);
      out = make_float4(0.0f, kHitBack, 0.0f, __uint_as_float(encode_normal(0.0f, 1.0f, 0.0f)));
    }
    else
    {
      const float4 o = rays[2 * k], d = rays[2 * k + 1];
      const float s = __fmul_rn(0.9999995f, h.t);
      const float p[3] = {__fadd_rn(o.x, __fmul_rn(s, d.x)), __fadd_rn(o.y, __fmul_rn(s, d.y)),
                          __fadd_rn(o.z, __fmul_rn(s, d.z))};
      const FrameGeom g = geoms[h.geomId];
      const uint32_t ia = g.sortedIdx[3 * (size_t)h.primId + 0];
      const uint32_t ib = g.sortedIdx[3 * (size_t)h.primId + 1];
      const uint32_t ic = g.sortedIdx[3 * (size_t)h.primId + 2];
      const float4 A = g.verts[ia], B = g.verts[ib], C = g.verts[ic];
      const float e1[3] = {__fsub_rn(B.x, A.x), __fsub_rn(B.y, A.y), __fsub_rn(B.z, A.z)};
      const float e2[3] = {__fsub_rn(C.x, A.x), __fsub_rn(C.y, A.y), __fsub_rn(C.z, A.z)};
      const float tn0[3] = {__fsub_rn(__fmul_rn(e1[1], e2[2]), __fmul_rn(e1[2], e2[1])),
                            __fsub_rn(__fmul_rn(e1[2], e2[0]), __fmul_rn(e1[0], e2[2])),
                            __fsub_rn(__fmul_rn(e1[0], e2[1]), __fmul_rn(e1[1], e2[0]))};
      const float4 nA = g.normals[ia], nB = g.normals[ib], nC = g.normals[ic];
      const float u = h.coords[0], v = h.coords[1];
      const float w0 = __fsub_rn(__fsub_rn(1.0f, u), v);
      const float hn0[3] = {__fadd_rn(__fadd_rn(__fmul_rn(w0, nA.x), __fmul_rn(v, nB.x)), __fmul_rn(u, nC.x)),
                            __fadd_rn(__fadd_rn(__fmul_rn(w0, nA.y), __fmul_rn(v, nB.y)), __fmul_rn(u, nC.y)),
                            __fadd_rn(__fadd_rn(__fmul_rn(w0, nA.z), __fmul_rn(v, nB.z)), __fmul_rn(u, nC.z))};
      const float* M = normMatrices + 16 * (size_t)h.instId;
      float hn[3], tn[3];
      mul3x3(M, hn0, hn);
      hrt::rg::normalize3(hn);
      mul3x3(M, tn0, tn);
      hrt::rg::normalize3(tn);
      if (hrt::rg::dot3(tn, hn) < 0.0f)
      {
        hn[0] = __fmul_rn(hn[0], -1.0f);
        hn[1] = __fmul_rn(hn[1], -1.0f);
        hn[2] = __fmul_rn(hn[2], -1.0f);
      }
      const float dd[3] = {d.x, d.y, d.z};
      const float flip = hrt::rg::dot3(dd, tn) > 1e-5f ? -1.0f : 1.0f;
      const uint32_t e = encode_normal(__fmul_rn(hn[0], flip), __fmul_rn(hn[1], flip), __fmul_rn(hn[2], flip));
      out = make_float4(p[0], p[1], p[2], __uint_as_float(e));
    }
    positions[pixel[k]] = out;
    flag[k] = out.y < kHitBack ? 1 : 0;
  }
}

// Flagged rays per block of kThreads * kChunk traced rays.
__global__ void __launch_bounds__(kThreads) k_flag_count(const uint8_t* __restrict__ flag, uint64_t n,
                                                         uint32_t* __restrict__ blockCount)
{
  __shared__ uint32_t s_warp[kThreads / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kThreads * kChunk;
  uint32_t c = 0;
#pragma unroll
  for (int j = 0; j < kChunk; j++)
  {
    const uint64_t k = base + (uint64_t)j * kThreads + threadIdx.x;
    c += (k < n && flag[k]) ? 1u : 0u;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, o);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    uint32_t t = 0;
    for (int w = 0; w < kThreads / 32; w++) t += s_warp[w];
    blockCount[blockIdx.x] = t;
  }
}

// Exclusive scan of the block counts in one block; the total -> *total.
__global__ void __launch_bounds__(1024) k_scan_counts(uint32_t* blockCount, uint32_t nBlocks, unsigned long long* total)
{
  __shared__ uint32_t s[1024];
  __shared__ unsigned long long s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (uint32_t b0 = 0; b0 < nBlocks; b0 += 1024)
  {
    const uint32_t b = b0 + threadIdx.x;
    const uint32_t v = b < nBlocks ? blockCount[b] : 0u;
    s[threadIdx.x] = v;
    __syncthreads();
    for (uint32_t o = 1; o < 1024; o <<= 1)
    {
      const uint32_t y = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
      __syncthreads();
      s[threadIdx.x] += y;
      __syncthreads();
    }
    if (b < nBlocks) blockCount[b] = (uint32_t)s_carry + s[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) s_carry += s[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = s_carry;
}

// Pixel of every AO slot: the flagged traced rays, ranked in trace order
// (block offsets from k_scan_counts, ranks inside a block by warp ballots).
__global__ void __launch_bounds__(kThreads)
    k_rtao_slots(const uint8_t* __restrict__ flag, uint64_t n, const uint32_t* __restrict__ blockOffset,
                 const uint32_t* __restrict__ pixel, uint32_t* __restrict__ aoPixel, uint64_t slotCapacity,
                 uint32_t* errorWord)
{
  __shared__ uint32_t s_warp[kThreads / 32 + 1];
  const uint64_t base = (uint64_t)blockIdx.x * kThreads * kChunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t run = 0;
  for (int j = 0; j < kChunk; j++)
  {
    const uint64_t k = base + (uint64_t)j * kThreads + threadIdx.x;
    const bool f = k < n && flag[k];
    const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, f);
    if (lane == 0) s_warp[warp] = __popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0)
    {
      uint32_t t = 0;
      for (int w = 0; w < kThreads / 32; w++)
      {
        const uint32_t c = s_warp[w];
        s_warp[w] = t;
        t += c;
      }
      s_warp[kThreads / 32] = t;
    }
    __syncthreads();
    const uint64_t slot = (uint64_t)blockOffset[blockIdx.x] + run + s_warp[warp] + __popc(ballot & ((1u << lane) - 1u));
    run += s_warp[kThreads / 32];
    __syncthreads();
    if (!f) continue;
    if (slot >= slotCapacity)
    {
      atomicOr(errorWord, kErrLayout);
      continue;
    }
    aoPixel[slot] = pixel[k];
  }
}

// The per-pixel part of kernel_InitAORay (examples/02_rtao/rtao.cpp:147-165),
// once per slot: the packed normal decoded (decodeNormal,
// examples/render_common.h:126-137), CoordinateSystem's frame about it
// (:38-54, the second branch's division in double as the renderer's
// unqualified sqrt makes it), the offset size epsilonOfPos (:96-98) and the
// pixel's row of the sample tile.  Record: {pos, eps}, {normal, invSign},
// {nx, tile row}, {ny, 0}.
__global__ void __launch_bounds__(kThreads)
    k_rtao_frames(const uint32_t* __restrict__ aoPixel, uint64_t slots, const float4* __restrict__ positions,
                  uint32_t width, uint32_t raysPerPixel, float4* __restrict__ frames)
{
  for (uint64_t s = (uint64_t)blockIdx.x * kThreads + threadIdx.x; s < slots; s += (uint64_t)gridDim.x * kThreads)
  {
    const uint32_t pix = aoPixel[s];
    const uint32_t x = pix % width, y = pix / width;
    const float4 pos = positions[pix];
    const uint32_t a = __float_as_uint(pos.w);
    const uint32_t ex = a & 0x0000FFFFu, ey = (a & 0xFFFF0000u) >> 16;
    const float sign = (ex & 1u) != 0 ? -1.0f : 1.0f;
    const float kInv = __fdiv_rn(1.0f, 32767.0f);
    float nrm[3];
    nrm[0] = __fmul_rn((float)(int16_t)(uint16_t)(ex & 0xfffeu), kInv);
    nrm[1] = __fmul_rn((float)(int16_t)(uint16_t)(ey & 0xffffu), kInv);
    const float zz = __fsub_rn(__fsub_rn(1.0f, __fmul_rn(nrm[0], nrm[0])), __fmul_rn(nrm[1], nrm[1]));
    nrm[2] = __fmul_rn(sign, __fsqrt_rn(zz < 0.0f ? 0.0f : zz));
    float nx[3];
    if (fabsf(nrm[0]) > fabsf(nrm[1]))
    {
      const float invLen = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(__fmul_rn(nrm[0], nrm[0]), __fmul_rn(nrm[2], nrm[2]))));
      nx[0] = __fmul_rn(__fmul_rn(-1.0f, nrm[2]), invLen);
      nx[1] = 0.0f;
      nx[2] = __fmul_rn(nrm[0], invLen);
    }
    else
    {
      const float s2 = __fadd_rn(__fmul_rn(nrm[1], nrm[1]), __fmul_rn(nrm[2], nrm[2]));
      const float invLen = __double2float_rn(__ddiv_rn(1.0, __dsqrt_rn((double)s2)));
      nx[0] = 0.0f;
      nx[1] = __fmul_rn(nrm[2], invLen);
      nx[2] = __fmul_rn(__fmul_rn(-1.0f, nrm[1]), invLen);
    }
    const float ny[3] = {__fsub_rn(__fmul_rn(nrm[1], nx[2]), __fmul_rn(nrm[2], nx[1])),
                         __fsub_rn(__fmul_rn(nrm[2], nx[0]), __fmul_rn(nrm[0], nx[2])),
                         __fsub_rn(__fmul_rn(nrm[0], nx[1]), __fmul_rn(nrm[1], nx[0]))};
    const float invSign = hrt::rg::dot3(nrm, nrm) > 0.0f ? 1.0f : -1.0f;
    // std::max(a, b) = a < b ? b : a
    const float ax = fabsf(pos.x), ay = fabsf(pos.y), az = fabsf(pos.z);
    const float myz = ay < az ? az : ay;
    const float mxyz = ax < myz ? myz : ax;
    const float gEps = 2e-5f, twoGEps = __fmul_rn(2.0f, gEps);
    const float eps = __fmul_rn(mxyz < twoGEps ? twoGEps : mxyz, gEps);
    const uint32_t tileRow = ((y % kAoTile) * kAoTile + (x % kAoTile)) * raysPerPixel;
    float4* o = frames + 4 * s;
    o[0] = make_float4(pos.x, pos.y, pos.z, eps);
    o[1] = make_float4(nrm[0], nrm[1], nrm[2], invSign);
    o[2] = make_float4(nx[0], nx[1], nx[2], __uint_as_float(tileRow));
    o[3] = make_float4(ny[0], ny[1], ny[2], 0.0f);
  }
}

// The per-ray part of kernel_InitAORay: one thread per AO ray (slot s, sample
// z at s * raysPerPixel + z), MapSampleToCosineDistribution with the tile
// entry's sample direction (dev: (sinT cosP, sinT sinP, cosT) per entry) and
// OffsRayPos (examples/render_common.h:56-112).  Consecutive threads write
// consecutive rays.
__global__ void __launch_bounds__(kThreads)
    k_rtao_ao_rays(const float4* __restrict__ frames, uint64_t nRays, uint32_t raysPerPixel,
                   const float4* __restrict__ dev, float aoMaxRadius, float4* __restrict__ aoRays)
{
  for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < nRays; i += (uint64_t)gridDim.x * kThreads)
  {
    const uint64_t s = i / raysPerPixel;
    const uint32_t z = (uint32_t)(i - s * raysPerPixel);
    const float4* fr = frames + 4 * s;
    const float4 P = fr[0], N = fr[1], X = fr[2], Y = fr[3];
    const float nrm[3] = {N.x, N.y, N.z}, nx[3] = {X.x, X.y, X.z}, ny[3] = {Y.x, Y.y, Y.z};
    const float4 dv = dev[__float_as_uint(X.w) + z];
    float res[3];
#pragma unroll
    for (int c = 0; c < 3; c++)
      res[c] = __fadd_rn(__fadd_rn(__fmul_rn(nx[c], dv.x), __fmul_rn(ny[c], dv.y)), __fmul_rn(nrm[c], dv.z));
    if (__fmul_rn(N.w, hrt::rg::dot3(res, nrm)) < 0.0f)
    {
#pragma unroll
      for (int c = 0; c < 3; c++)
        res[c] = __fsub_rn(__fadd_rn(__fmul_rn(__fmul_rn(-1.0f, nx[c]), dv.x), __fmul_rn(ny[c], dv.y)),
                           __fmul_rn(nrm[c], dv.z));
    }
    const float se = __fmul_rn(hrt::rg::dot3(res, nrm) < 0.0f ? -1.0f : 1.0f, P.w);
    aoRays[2 * i + 0] = make_float4(__fadd_rn(P.x, __fmul_rn(se, nrm[0])), __fadd_rn(P.y, __fmul_rn(se, nrm[1])),
                                    __fadd_rn(P.z, __fmul_rn(se, nrm[2])), 0.0f);
    aoRays[2 * i + 1] = make_float4(res[0], res[1], res[2], aoMaxRadius);
  }
}

// kernel_TraceAORay summed over the samples + kernel_AO2Color
// (examples/02_rtao/rtao.cpp:62-73,167-185), one thread per pixel with a hit.
__global__ void __launch_bounds__(kThreads)
    k_rtao_colors(const uint8_t* __restrict__ aoHit, const uint32_t* __restrict__ aoPixel, uint64_t slots,
                  uint32_t raysPerPixel, float power, float* __restrict__ visibility, uint32_t* __restrict__ colors)
{
  for (uint64_t s = (uint64_t)blockIdx.x * kThreads + threadIdx.x; s < slots; s += (uint64_t)gridDim.x * kThreads)
  {
    float vis = 0.0f;
    for (uint32_t z = 0; z < raysPerPixel; z++) vis = __fadd_rn(vis, aoHit[s * raysPerPixel + z] ? 0.0f : 1.0f);
    const float normCoeff = __fdiv_rn(1.0f, (float)raysPerPixel);
    const float a = __fmul_rn(vis, normCoeff);
    const float res = power == 1.0f ? a : powf(a, power);
    const float c = (res > 0.0f ? res : 0.0f);
    const int g = f2i(__fmul_rn(c < 1.0f ? c : 1.0f, 255.0f));
    const uint32_t pix = aoPixel[s];
    visibility[pix] = vis;
    colors[pix] = (uint32_t)g + ((uint32_t)g << 8) + ((uint32_t)g << 16) + (255u << 24);
  }
}

uint32_t grid_for(uint64_t n, int numSMs)
{
  uint64_t g = (n + kThreads - 1) / kThreads;
  const uint64_t cap = (uint64_t)numSMs * 16;
  return (uint32_t)(g < 1 ? 1 : (g > cap ? cap : g));
}

// ---------------------------------------------------------------- host: sample tile
// Niederreiter base-2 direction numbers, 4 dimensions x 31 bits, as the
// renderer's initQuasirandomGenerator computes them
// (core/common/qmc_sobol_niederreiter.cpp:13-186; Bratley, Fox and Niederreiter,
// ACM TOMACS 2(3), 1992).  Polynomials over GF(2) are bit masks (bit k = x^k).
int gf2_degree(uint64_t p)
{
  int d = 63;
  while (d > 0 && !((p >> d) & 1u)) d--;
  return d;
}

uint64_t gf2_mul(uint64_t a, uint64_t b)
{
  uint64_t r = 0;
  for (int k = 0; k < 64; k++)
    if ((b >> k) & 1u) r ^= a << k;
  return r;
}

bool gf2_divides(uint64_t d, uint64_t p)
{
  const int dd = gf2_degree(d);
  while (p != 0 && gf2_degree(p) >= dd) p ^= d << (gf2_degree(p) - dd);
  return p == 0;
}

void qmc_directions(uint32_t table[4][31])
{
  // the first four irreducible polynomials in numeric order, found as the
  // reference does: trial division by the ones found before
  uint64_t poly[4] = {2u, 0u, 0u, 0u};
  for (int n = 1; n < 4; n++)
    for (uint64_t p = poly[n - 1] + 1;; p++)
    {
      bool irreducible = true;
      for (int k = 0; k < n; k++) irreducible = irreducible && !gf2_divides(poly[k], p);
      if (irreducible)
      {
        poly[n] = p;
        break;
      }
    }
  for (int d = 0; d < 4; d++)
  {
    const int e = gf2_degree(poly[d]);
    for (int i = 0; i < 31; i++) table[d][i] = 0u;
    uint64_t power = 1u;  // poly^(q+1) for output bits q*e .. q*e+e-1
    for (int r = 0; r < 31; r++)
    {
      const int u = r % e;
      if (u == 0) power = gf2_mul(power, poly[d]);
      const int m = gf2_degree(power), m1 = m - e;
      // v: m1 zeros, then ones up to m, then the recurrence whose characteristic
      // polynomial is `power`: v[i] = sum_k coefficient(x^(m-k)) v[i-k]
      uint8_t v[31 + 64];
      for (int i = 0; i < 31 + e; i++)
      {
        if (i < m) v[i] = i < m1 ? 0 : 1;
        else
        {
          uint8_t s = 0;
          for (int k = 1; k <= m; k++) s ^= (uint8_t)(((power >> (m - k)) & 1u) & v[i - k]);
          v[i] = s;
        }
      }
      for (int i = 0; i < 31; i++) table[d][i] |= (uint32_t)v[i + u] << (30 - r);
    }
  }
}

}  // namespace

struct hrt_frame
{
  hrt_context* ctx = nullptr;
  // eye pass, one entry per traced ray / pixel
  float4*   rays = nullptr;
  uint32_t* pixel = nullptr;
  hrt_hit*  hits = nullptr;
  float4*   positions = nullptr;
  uint8_t*  flag = nullptr;
  float*    visibility = nullptr;
  uint32_t* blockCount = nullptr;
  uint64_t  pixCap = 0, blockCap = 0;
  // AO pass
  float4*   aoRays = nullptr;
  uint32_t* aoPixel = nullptr;
  float4*   frames = nullptr;  // per slot: the pixel's AO frame (k_rtao_frames)
  uint8_t*  aoHit = nullptr;
  uint64_t  slotCap = 0, aoCap = 0;
  // sample tile: sample directions per entry
  float4*   dev = nullptr;
  uint32_t  raysPerPixel = 0;
  // per geometry vertex normals
  std::vector<float4*>  normals;
  std::vector<uint64_t> normalCount;
  FrameGeom*            dGeoms = nullptr;
  uint32_t              geomCap = 0;
  float*                dNormMat = nullptr;
  uint32_t              normMatCap = 0;
  // small state: total (u64) + error word, device and pinned host
  unsigned long long* dTotal = nullptr;
  unsigned long long* hTotal = nullptr;
  // colours for a destination in pageable host memory
  uint32_t* colorBuf = nullptr;
  uint64_t  colorCap = 0;
  // last frame
  uint64_t lastPixels = 0, lastSlots = 0;
  uint32_t lastRaysPerPixel = 0;
};

namespace
{

int grow(hrt_context* ctx, void** p, uint64_t bytes)
{
  if (*p) cudaFree(*p);
  *p = nullptr;
  HRT_CUDA(ctx, cudaMalloc(p, bytes ? bytes : 16));
  return HRT_OK;
}

int ensure_pixels(hrt_frame* f, uint64_t n)
{
  if (n <= f->pixCap) return HRT_OK;
  hrt_context* ctx = f->ctx;
  int st = HRT_OK;
  if ((st = grow(ctx, (void**)&f->rays, 32 * n)) || (st = grow(ctx, (void**)&f->pixel, 4 * n)) ||
      (st = grow(ctx, (void**)&f->hits, sizeof(hrt_hit) * n)) || (st = grow(ctx, (void**)&f->positions, 16 * n)) ||
      (st = grow(ctx, (void**)&f->flag, n)) || (st = grow(ctx, (void**)&f->visibility, 4 * n)))
  {
    f->pixCap = 0;
    return st;
  }
  f->pixCap = n;
  const uint64_t blocks = (n + kThreads * kChunk - 1) / (kThreads * kChunk);
  if (blocks > f->blockCap)
  {
    if ((st = grow(ctx, (void**)&f->blockCount, 4 * blocks))) return st;
    f->blockCap = blocks;
  }
  return HRT_OK;
}

// Where the kernels write a frame's colours: device or managed memory
// directly (4-byte aligned); host memory (page-locked or not) and unaligned
// arrays through the frame's own buffer and one copy at the end of the frame.
int color_target(hrt_frame* f, uint32_t* colors, uint64_t n, uint32_t** target)
{
  cudaPointerAttributes a;
  if (aligned_to(colors, 4) && cudaPointerGetAttributes(&a, colors) == cudaSuccess &&
      (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged))
  {
    *target = colors;
    return HRT_OK;
  }
  cudaGetLastError();  // an unregistered pointer may leave an error behind
  if (n > f->colorCap)
  {
    f->colorCap = 0;
    const int st = grow(f->ctx, (void**)&f->colorBuf, 4 * n);
    if (st) return st;
    f->colorCap = n;
  }
  *target = f->colorBuf;
  return HRT_OK;
}

int finish_colors(hrt_frame* f, uint32_t* colors, const uint32_t* target, uint64_t n, cudaStream_t cs)
{
  if (target == colors) return HRT_OK;
  HRT_CUDA(f->ctx, cudaMemcpyAsync(colors, target, 4 * n, cudaMemcpyDefault, cs));
  HRT_CUDA(f->ctx, cudaStreamSynchronize(cs));
  return HRT_OK;
}

int check_scene(hrt_scene* s)
{
  if (!s->committed) return fail(s->ctx, HRT_ERR_STATE, "frame before hrt_commit_scene");
  return HRT_OK;
}

}  // namespace

extern "C" {

int hrt_rtao_qmc_table(uint32_t* table)
{
  if (!table) return HRT_ERR_INVALID_ARGUMENT;
  uint32_t t[4][31];
  qmc_directions(t);
  std::memcpy(table, t, sizeof(t));
  return HRT_OK;
}

int hrt_rtao_qmc_tile(uint32_t raysPerPixel, float* tile)
{
  if (!tile || raysPerPixel == 0 || raysPerPixel > HRT_MAX_AO_RAYS_PER_PIXEL) return HRT_ERR_INVALID_ARGUMENT;
  uint32_t t[4][31];
  qmc_directions(t);
  auto sample = [&](uint32_t pos, int dim) {  // rndQmcSobolN (qmc_sobol_niederreiter.h:11-20)
    uint32_t r = 0;
    for (int bit = 0; bit < 31; bit++, pos >>= 1)
      if (pos & 1u) r ^= t[dim][bit];
    return (float)(r + 1u) * (1.0f / 2147483648.0f);
  };
  const size_t n = (size_t)kAoTile * kAoTile * raysPerPixel;
  std::memset(tile, 0, sizeof(float) * 2 * n);
  std::vector<uint32_t> filled((size_t)kAoTile * kAoTile, 0u);
  for (size_t i = 0; i < n; i++)
  {
    int ix = (int)(sample((uint32_t)i, 0) * (float)kAoTile);
    int iy = (int)(sample((uint32_t)i, 1) * (float)kAoTile);
    if (ix >= (int)kAoTile) ix = kAoTile - 1;
    if (iy >= (int)kAoTile) iy = kAoTile - 1;
    const size_t cell = (size_t)iy * kAoTile + (size_t)ix;
    if (filled[cell] < raysPerPixel)
    {
      float* o = tile + 2 * (cell * raysPerPixel + filled[cell]++);
      o[0] = sample((uint32_t)i, 2);
      o[1] = sample((uint32_t)i, 3);
    }
  }
  return HRT_OK;
}

int hrt_frame_create(hrt_context* ctx, hrt_frame** out)
{
  if (!ctx || !out) return HRT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  cudaSetDevice(ctx->device);
  hrt_frame* f = new hrt_frame();
  f->ctx = ctx;
  cudaError_t e = cudaMalloc((void**)&f->dTotal, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&f->hTotal, 2 * sizeof(unsigned long long));
  if (e != cudaSuccess)
  {
    hrt_frame_destroy(f);
    return cuda_fail(ctx, e, "frame state");
  }
  *out = f;
  return HRT_OK;
}

int hrt_frame_destroy(hrt_frame* f)
{
  if (!f) return HRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(f->ctx->device);
  void* dev[] = {f->rays, f->pixel, f->hits, f->positions, f->flag, f->visibility, f->blockCount, f->aoRays,
                 f->aoPixel, f->aoHit, f->dev, f->dGeoms, f->dNormMat, f->dTotal, f->colorBuf, f->frames};
  for (void* p : dev)
    if (p) cudaFree(p);
  for (float4* p : f->normals)
    if (p) cudaFree(p);
  if (f->hTotal) cudaFreeHost(f->hTotal);
  delete f;
  return HRT_OK;
}

int hrt_frame_set_ao_tile(hrt_frame* f, const float* tile, uint32_t raysPerPixel)
{
  if (!f || !tile || raysPerPixel == 0 || raysPerPixel > HRT_MAX_AO_RAYS_PER_PIXEL) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = f->ctx;
  cudaSetDevice(ctx->device);
  const size_t n = (size_t)kAoTile * kAoTile * raysPerPixel;
  // MapSampleToCosineDistribution's sample-only part (examples/render_common.h:58-72),
  // power 1 as kernel_InitAORay passes it, in the renderer's types: the float
  // angle 2 pi r1 and the float arguments of pow and sqrt go through the double
  // functions; the products are float
  std::vector<float4> dv(n);
  const float twoPi = 6.28318530717958647692f;
  for (size_t i = 0; i < n; i++)
  {
    const float r1 = tile[2 * i], r2 = tile[2 * i + 1];
    const float phi = twoPi * r1;
    const float sinPhi = (float)std::sin((double)phi);
    const float cosPhi = (float)std::cos((double)phi);
    const float cosTheta = (float)std::pow((double)(1.0f - r2), (double)(1.0f / (1.0f + 1.0f)));
    const float sinTheta = (float)std::sqrt((double)(1.0f - cosTheta * cosTheta));
    dv[i] = make_float4(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta, 0.0f);
  }
  if (f->dev) cudaFree(f->dev);
  f->dev = nullptr;
  f->raysPerPixel = 0;
  HRT_CUDA(ctx, cudaMalloc((void**)&f->dev, sizeof(float4) * n));
  HRT_CUDA(ctx, cudaMemcpy(f->dev, dv.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
  f->raysPerPixel = raysPerPixel;
  return HRT_OK;
}

int hrt_frame_set_normals(hrt_frame* f, uint32_t geomId, const float* normals, uint64_t nVerts)
{
  if (!f || (!normals && nVerts)) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = f->ctx;
  cudaSetDevice(ctx->device);
  if (geomId >= f->normals.size())
  {
    f->normals.resize(geomId + 1, nullptr);
    f->normalCount.resize(geomId + 1, 0);
  }
  if (f->normals[geomId]) cudaFree(f->normals[geomId]);
  f->normals[geomId] = nullptr;
  f->normalCount[geomId] = 0;
  HRT_CUDA(ctx, cudaMalloc((void**)&f->normals[geomId], 16 * (nVerts ? nVerts : 1)));
  if (nVerts) HRT_CUDA(ctx, cudaMemcpy(f->normals[geomId], normals, 16 * nVerts, cudaMemcpyDefault));
  f->normalCount[geomId] = nVerts;
  return HRT_OK;
}

int hrt_frame_render_eye(hrt_frame* f, hrt_scene* s, const float projInv[16], const float worldViewInv[16],
                         uint32_t width, uint32_t height, uint32_t* colors, void* stream)
{
  if (!f || !s || !projInv || !worldViewInv || s->ctx != f->ctx) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = f->ctx;
  const uint64_t n = (uint64_t)width * height;
  if (n == 0) return HRT_OK;
  if (!colors) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "null colour buffer");
  if (width > 0xFFFFu || height > 0xFFFFu) return fail(ctx, HRT_ERR_CAPACITY, "image sides above 65535");
  int st = check_scene(s);
  if (st) return st;
  cudaSetDevice(ctx->device);
  if ((st = ensure_pixels(f, n))) return st;
  cudaStream_t cs = (cudaStream_t)stream;
  Mat4 p, v;
  std::memcpy(p.m, projInv, sizeof(p.m));
  std::memcpy(v.m, worldViewInv, sizeof(v.m));
  const int packed = (width % 8 == 0 && height % 8 == 0) ? 1 : 0;
  k_frame_eye_rays<<<grid_for(n, ctx->numSMs), kThreads, 0, cs>>>(p, v, width, height, packed, 0.0f, FLT_MAX, f->rays,
                                                                  f->pixel);
  HRT_CUDA(ctx, cudaGetLastError());
  if ((st = hrt_query_nearest(s, reinterpret_cast<const float*>(f->rays), n, f->hits, stream))) return st;
  uint32_t* out = nullptr;
  if ((st = color_target(f, colors, n, &out))) return st;
  k_eye_colors<<<grid_for(n, ctx->numSMs), kThreads, 0, cs>>>(f->hits, f->pixel, n, out);
  HRT_CUDA(ctx, cudaGetLastError());
  f->lastPixels = n;
  f->lastSlots = 0;
  f->lastRaysPerPixel = 0;
  return finish_colors(f, colors, out, n, cs);
}

int hrt_frame_render_rtao(hrt_frame* f, hrt_scene* s, const hrt_rtao_params* prm, const float* normMatrices,
                          uint32_t* colors, void* stream)
{
  if (!f || !s || !prm || s->ctx != f->ctx) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = f->ctx;
  const uint64_t n = (uint64_t)prm->width * prm->height;
  if (n == 0) return HRT_OK;
  if (!colors) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "null colour buffer");
  if (prm->width > 0xFFFFu || prm->height > 0xFFFFu) return fail(ctx, HRT_ERR_CAPACITY, "image sides above 65535");
  if (f->raysPerPixel == 0) return fail(ctx, HRT_ERR_STATE, "no AO sample tile (hrt_frame_set_ao_tile)");
  int st = check_scene(s);
  if (st) return st;
  const uint32_t nInst = (uint32_t)s->insts.size();
  if (nInst > 0 && !normMatrices) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "null normal matrices");
  // the geometries' device arrays with their normals
  std::vector<FrameGeom> hg(s->geoms.size());
  for (size_t g = 0; g < hg.size(); g++)
  {
    const Geom& G = s->geoms[g];
    if (G.nTris > 0 && (g >= f->normals.size() || !f->normals[g] || f->normalCount[g] != G.nVerts))
      return fail(ctx, HRT_ERR_STATE, "geometry " + std::to_string(g) + " has no vertex normals of its vertex count");
    hg[g] = FrameGeom{G.verts, G.sortedIdx, g < f->normals.size() ? f->normals[g] : nullptr, G.nTris};
  }
  cudaSetDevice(ctx->device);
  if ((st = ensure_pixels(f, n))) return st;
  if (hg.size() > f->geomCap)
  {
    if ((st = grow(ctx, (void**)&f->dGeoms, sizeof(FrameGeom) * hg.size()))) return st;
    f->geomCap = (uint32_t)hg.size();
  }
  if (nInst > f->normMatCap)
  {
    if ((st = grow(ctx, (void**)&f->dNormMat, 64 * (uint64_t)nInst))) return st;
    f->normMatCap = nInst;
  }
  cudaStream_t cs = (cudaStream_t)stream;
  if (!hg.empty())
    HRT_CUDA(ctx, cudaMemcpyAsync(f->dGeoms, hg.data(), sizeof(FrameGeom) * hg.size(), cudaMemcpyHostToDevice, cs));
  if (nInst) HRT_CUDA(ctx, cudaMemcpyAsync(f->dNormMat, normMatrices, 64 * (size_t)nInst, cudaMemcpyHostToDevice, cs));
  HRT_CUDA(ctx, cudaMemsetAsync(f->dTotal, 0, 2 * sizeof(unsigned long long), cs));
  uint32_t* dErr = reinterpret_cast<uint32_t*>(f->dTotal + 1);
  Mat4 p, v;
  std::memcpy(p.m, prm->projInv, sizeof(p.m));
  std::memcpy(v.m, prm->worldViewInv, sizeof(v.m));
  const int packed = (prm->width % 8 == 0 && prm->height % 8 == 0) ? 1 : 0;
  const uint32_t grid = grid_for(n, ctx->numSMs);
  k_frame_eye_rays<<<grid, kThreads, 0, cs>>>(p, v, prm->width, prm->height, packed, prm->zNear, prm->zFar, f->rays,
                                              f->pixel);
  HRT_CUDA(ctx, cudaGetLastError());
  if ((st = hrt_query_nearest(s, reinterpret_cast<const float*>(f->rays), n, f->hits, stream))) return st;
  k_rtao_positions<<<grid, kThreads, 0, cs>>>(f->rays, f->hits, f->pixel, n, f->dGeoms, (uint32_t)hg.size(),
                                              f->dNormMat, nInst, f->positions, f->flag, dErr);
  const uint32_t nBlocks = (uint32_t)((n + kThreads * kChunk - 1) / (kThreads * kChunk));
  k_flag_count<<<nBlocks, kThreads, 0, cs>>>(f->flag, n, f->blockCount);
  k_scan_counts<<<1, 1024, 0, cs>>>(f->blockCount, nBlocks, f->dTotal);
  HRT_CUDA(ctx, cudaGetLastError());
  HRT_CUDA(ctx, cudaMemcpyAsync(f->hTotal, f->dTotal, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, cs));
  HRT_CUDA(ctx, cudaStreamSynchronize(cs));
  const uint64_t slots = f->hTotal[0];
  if ((uint32_t)f->hTotal[1] & kErrIndexRange)
    return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "a hit names a geometry, instance or triangle out of range");
  const uint32_t R = f->raysPerPixel;
  const uint64_t nAo = slots * R;
  if (nAo > 0xFFFFFFFFull) return fail(ctx, HRT_ERR_CAPACITY, "more than 2^32-1 AO rays in one frame");
  if (slots > f->slotCap)
  {
    f->slotCap = 0;
    if ((st = grow(ctx, (void**)&f->aoPixel, 4 * slots)) || (st = grow(ctx, (void**)&f->frames, 64 * slots)))
      return st;
    f->slotCap = slots;
  }
  if (nAo > f->aoCap)
  {
    f->aoCap = 0;
    if ((st = grow(ctx, (void**)&f->aoRays, 32 * nAo)) || (st = grow(ctx, (void**)&f->aoHit, nAo))) return st;
    f->aoCap = nAo;
  }
  uint32_t* out = nullptr;
  if ((st = color_target(f, colors, n, &out))) return st;
  HRT_CUDA(ctx, cudaMemsetAsync(out, 0, 4 * n, cs));
  HRT_CUDA(ctx, cudaMemsetAsync(f->visibility, 0, 4 * n, cs));
  if (slots > 0)
  {
    k_rtao_slots<<<nBlocks, kThreads, 0, cs>>>(f->flag, n, f->blockCount, f->pixel, f->aoPixel, f->slotCap, dErr);
    k_rtao_frames<<<grid_for(slots, ctx->numSMs), kThreads, 0, cs>>>(f->aoPixel, slots, f->positions, prm->width, R,
                                                                     f->frames);
    k_rtao_ao_rays<<<grid_for(nAo, ctx->numSMs), kThreads, 0, cs>>>(f->frames, nAo, R, f->dev, prm->aoMaxRadius,
                                                                    f->aoRays);
    HRT_CUDA(ctx, cudaGetLastError());
    if ((st = hrt_query_any(s, reinterpret_cast<const float*>(f->aoRays), nAo, f->aoHit, stream))) return st;
    k_rtao_colors<<<grid_for(slots, ctx->numSMs), kThreads, 0, cs>>>(f->aoHit, f->aoPixel, slots, R, prm->power,
                                                                     f->visibility, out);
    HRT_CUDA(ctx, cudaGetLastError());
  }
  f->lastPixels = n;
  f->lastSlots = slots;
  f->lastRaysPerPixel = R;
  return finish_colors(f, colors, out, n, cs);
}

int hrt_frame_get_buffer(const hrt_frame* f, int which, const void** data, uint64_t* count)
{
  if (!f || !data || !count) return HRT_ERR_INVALID_ARGUMENT;
  const uint64_t n = f->lastPixels, slots = f->lastSlots, ao = slots * f->lastRaysPerPixel;
  switch (which)
  {
    case HRT_FRAME_EYE_RAYS: *data = f->rays; *count = n; break;
    case HRT_FRAME_RAY_PIXEL: *data = f->pixel; *count = n; break;
    case HRT_FRAME_EYE_HITS: *data = f->hits; *count = n; break;
    case HRT_FRAME_POSITIONS: *data = f->positions; *count = f->lastRaysPerPixel ? n : 0; break;
    case HRT_FRAME_VISIBILITY: *data = f->visibility; *count = f->lastRaysPerPixel ? n : 0; break;
    case HRT_FRAME_AO_RAYS: *data = f->aoRays; *count = ao; break;
    case HRT_FRAME_AO_PIXEL: *data = f->aoPixel; *count = slots; break;
    case HRT_FRAME_AO_HITS: *data = f->aoHit; *count = ao; break;
    default: return HRT_ERR_INVALID_ARGUMENT;
  }
  return HRT_OK;
}

int hrt_frame_read_buffer(const hrt_frame* f, int which, void* dst, uint64_t capacityBytes, uint64_t* bytes)
{
  if (!f || !bytes) return HRT_ERR_INVALID_ARGUMENT;
  const void* src = nullptr;
  uint64_t count = 0;
  const int st = hrt_frame_get_buffer(f, which, &src, &count);
  if (st) return st;
  static const uint64_t kEntryBytes[] = {32, 4, sizeof(hrt_hit), 16, 4, 4, 32, 1};
  *bytes = count * kEntryBytes[which];
  if (*bytes == 0) return HRT_OK;
  if (!dst || capacityBytes < *bytes) return fail(f->ctx, HRT_ERR_CAPACITY, "frame buffer larger than the destination");
  cudaSetDevice(f->ctx->device);
  HRT_CUDA(f->ctx, cudaDeviceSynchronize());
  HRT_CUDA(f->ctx, cudaMemcpy(dst, src, *bytes, cudaMemcpyDefault));
  return HRT_OK;
}

}  // extern "C"
