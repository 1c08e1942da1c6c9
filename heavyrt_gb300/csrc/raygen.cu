// Ray generation on the device, so that a frame's eye rays and the ambient-
// occlusion rays chained from their hits never cross the host link.
//
//  * k_eye_rays: HeavyRT's renderer eye rays, RTAO::kernel_InitEyeRay
//    (examples/02_rtao/rtao.cpp:133-144; examples/01_eye_rays/eye_ray.cpp:26-47)
//    with EyeRayDirNormalized and transform_ray3f (examples/render_common.h:6-36):
//    inverse projection and world-view matrices, one ray per pixel centre.
//    Float arithmetic in the reference's order with explicit round-to-nearest
//    operations (mat x vec sums ((m0 x + m1 y) + m2 z) + m3 w, normalize(v) =
//    v * (1 / sqrt(dot(v, v)))), so the rays equal the host restatement bit for bit.
//  * k_pinhole_rays / k_ao_*: the benchmark's camera and its cosine-weighted
//    AO rays (Malley's method on the seeded PCG32 streams of
//    heavyrt_gb300/csrc/workload.c): correctly rounded float operations in the
//    host generator's order, so the rays are the host generator's bit for bit.
#include <cmath>
#include <cstring>
#include <vector>

#include "hrt_internal.cuh"
#include "raygen_common.cuh"

using namespace hrt;
using namespace hrt::api;

namespace
{

constexpr int kThreads = 256;

// ---------------------------------------------------------------- renderer eye rays
using hrt::rg::Mat4;

__global__ void __launch_bounds__(kThreads) k_eye_rays(Mat4 projInv, Mat4 worldViewInv, uint32_t width, uint32_t height,
                                                       float tNear, float tFar, float4* __restrict__ rays)
{
  const uint64_t n = (uint64_t)width * height;
  for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kThreads)
  {
    const uint32_t y = (uint32_t)(i / width), x = (uint32_t)(i % width);
    hrt::rg::eye_ray(projInv, worldViewInv, x, y, width, height, tNear, tFar, rays[2 * i + 0], rays[2 * i + 1]);
  }
}

// ---------------------------------------------------------------- benchmark camera
struct Pinhole
{
  float f[3], rgt[3], up[3];
  float th, aspect;
  float eye[3];
};

// each component divided by the length (the host generator's wl_normf)
__device__ __forceinline__ void fnorm(float v[3])
{
  const float l = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(v[0], v[0]), __fmul_rn(v[1], v[1])), __fmul_rn(v[2], v[2])));
  v[0] = __fdiv_rn(v[0], l);
  v[1] = __fdiv_rn(v[1], l);
  v[2] = __fdiv_rn(v[2], l);
}

__global__ void __launch_bounds__(kThreads) k_pinhole_rays(Pinhole c, uint32_t width, uint32_t height, float tmin,
                                                           float tmax, float4* __restrict__ rays)
{
  const uint64_t n = (uint64_t)width * height;
  for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kThreads)
  {
    const uint32_t y = (uint32_t)(i / width), x = (uint32_t)(i % width);
    const float sx = __fmul_rn(
        __fmul_rn(__fsub_rn(__fdiv_rn(__fmul_rn(2.0f, __fadd_rn((float)x, 0.5f)), (float)width), 1.0f), c.th), c.aspect);
    const float sy =
        __fmul_rn(__fsub_rn(1.0f, __fdiv_rn(__fmul_rn(2.0f, __fadd_rn((float)y, 0.5f)), (float)height)), c.th);
    float d[3];
#pragma unroll
    for (int k = 0; k < 3; k++) d[k] = __fadd_rn(__fadd_rn(c.f[k], __fmul_rn(sx, c.rgt[k])), __fmul_rn(sy, c.up[k]));
    fnorm(d);
    rays[2 * i + 0] = make_float4(c.eye[0], c.eye[1], c.eye[2], tmin);
    rays[2 * i + 1] = make_float4(d[0], d[1], d[2], tmax);
  }
}

// ---------------------------------------------------------------- AO rays
// PCG32 (XSH-RR, 64-bit LCG), seeded like the host generator.
struct Pcg
{
  uint64_t state, inc;
};

__device__ __forceinline__ uint32_t pcg_next(Pcg& r)
{
  const uint64_t old = r.state;
  r.state = old * 6364136223846793005ULL + r.inc;
  const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  const uint32_t rot = (uint32_t)(old >> 59u);
  return (xs >> rot) | (xs << ((32u - rot) & 31u));
}

__device__ __forceinline__ void pcg_seed(Pcg& r, uint64_t seed, uint64_t stream)
{
  r.state = 0u;
  r.inc = (stream << 1u) | 1u;
  pcg_next(r);
  r.state += seed;
  pcg_next(r);
}

__device__ __forceinline__ float pcg_uniformf(Pcg& r) { return __fmul_rn((float)(pcg_next(r) >> 8), 1.0f / 16777216.0f); }

struct GeomPtr
{
  const float4*   verts;
  const uint32_t* sortedIdx;
  uint32_t        nTris;
};

__device__ __forceinline__ bool is_hit(const float4* hits, uint64_t i)
{
  return __float_as_uint(__ldg(hits + 2 * i).w) != 0xFFFFFFFFu;  // geomId
}

// Hits per block of kThreads * 4 eye rays.
__global__ void __launch_bounds__(kThreads) k_ao_count(const float4* __restrict__ hits, uint64_t nEye,
                                                       uint32_t* __restrict__ blockCount)
{
  __shared__ uint32_t s_warp[kThreads / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kThreads * 4;
  uint32_t c = 0;
#pragma unroll
  for (int k = 0; k < 4; k++)
  {
    const uint64_t i = base + (uint64_t)k * kThreads + threadIdx.x;
    c += (i < nEye && is_hit(hits, i)) ? 1u : 0u;
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

// Exclusive scan of the block counts (one block); total hits -> *total.
__global__ void __launch_bounds__(1024) k_ao_scan(uint32_t* blockCount, uint32_t nBlocks, unsigned long long* total)
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

// One thread per eye ray: a hit writes its perHit AO rays after the rays of
// the hits before it (eye-ray order), exactly as the host generator does.
__global__ void __launch_bounds__(kThreads) k_ao_emit(uint64_t seed, const float4* __restrict__ eye,
                                                      const float4* __restrict__ hits, uint64_t nEye,
                                                      const GeomPtr* __restrict__ geoms, uint32_t nGeoms,
                                                      const uint32_t* __restrict__ blockOffset, uint32_t perHit,
                                                      float length, float offset, float4* __restrict__ out,
                                                      uint32_t* __restrict__ owner, uint64_t capacity,
                                                      uint32_t* errorWord)
{
  __shared__ uint32_t s_warp[kThreads / 32 + 1];
  const uint64_t base = (uint64_t)blockIdx.x * kThreads * 4;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t run = 0;  // hits of this block before the current chunk
  for (int k = 0; k < 4; k++)
  {
    const uint64_t i = base + (uint64_t)k * kThreads + threadIdx.x;
    const bool h = i < nEye && is_hit(hits, i);
    const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, h);
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
    if (!h) continue;
    const float4 hr0 = hits[2 * i];
    const float t = hr0.x;
    const uint32_t prim = __float_as_uint(hr0.y), gid = __float_as_uint(hr0.w);
    if (gid >= nGeoms || prim >= geoms[gid].nTris)
    {
      atomicOr(errorWord, kErrIndexRange);
      continue;
    }
    const float4 po = eye[2 * i], di = eye[2 * i + 1];
    const float p[3] = {__fadd_rn(po.x, __fmul_rn(t, di.x)), __fadd_rn(po.y, __fmul_rn(t, di.y)),
                        __fadd_rn(po.z, __fmul_rn(t, di.z))};
    const GeomPtr g = geoms[gid];
    const float4 A = g.verts[g.sortedIdx[3 * (size_t)prim + 0]];
    const float4 B = g.verts[g.sortedIdx[3 * (size_t)prim + 1]];
    const float4 C = g.verts[g.sortedIdx[3 * (size_t)prim + 2]];
    const float e1[3] = {__fsub_rn(B.x, A.x), __fsub_rn(B.y, A.y), __fsub_rn(B.z, A.z)};
    const float e2[3] = {__fsub_rn(C.x, A.x), __fsub_rn(C.y, A.y), __fsub_rn(C.z, A.z)};
    float n[3] = {__fsub_rn(__fmul_rn(e1[1], e2[2]), __fmul_rn(e1[2], e2[1])),
                  __fsub_rn(__fmul_rn(e1[2], e2[0]), __fmul_rn(e1[0], e2[2])),
                  __fsub_rn(__fmul_rn(e1[0], e2[1]), __fmul_rn(e1[1], e2[0]))};
    fnorm(n);
    const float facing = __fadd_rn(__fadd_rn(__fmul_rn(n[0], di.x), __fmul_rn(n[1], di.y)), __fmul_rn(n[2], di.z));
    if (facing > 0.0f)
    {
      n[0] = -n[0];
      n[1] = -n[1];
      n[2] = -n[2];
    }
    // orthonormal basis about n (Duff et al., "Building an Orthonormal Basis, Revisited", 2017)
    const float sgn = n[2] >= 0.0f ? 1.0f : -1.0f;
    const float aa = __fdiv_rn(-1.0f, __fadd_rn(sgn, n[2]));
    const float bb = __fmul_rn(__fmul_rn(n[0], n[1]), aa);
    const float tx[3] = {__fadd_rn(1.0f, __fmul_rn(__fmul_rn(__fmul_rn(sgn, n[0]), n[0]), aa)), __fmul_rn(sgn, bb),
                         -__fmul_rn(sgn, n[0])};
    const float ty[3] = {bb, __fadd_rn(sgn, __fmul_rn(__fmul_rn(n[1], n[1]), aa)), -n[1]};
    float o[3];
#pragma unroll
    for (int k2 = 0; k2 < 3; k2++) o[k2] = __fadd_rn(p[k2], __fmul_rn(offset, n[k2]));
    Pcg r;
    pcg_seed(r, seed, i + 16);
    for (uint32_t sIdx = 0; sIdx < perHit; sIdx++)
    {
      // Malley's method: a uniform point of the unit disk (rejection from the
      // square, at most 64 tries) lifted to the hemisphere
      float x = 0.0f, y = 0.0f, rr = 0.0f;
      for (int tries = 0; tries < 64; tries++)
      {
        x = __fsub_rn(__fmul_rn(2.0f, pcg_uniformf(r)), 1.0f);
        y = __fsub_rn(__fmul_rn(2.0f, pcg_uniformf(r)), 1.0f);
        rr = __fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y));
        if (rr <= 1.0f) break;
      }
      if (rr > 1.0f)
      {
        x = 0.0f;
        y = 0.0f;
        rr = 0.0f;
      }
      const float z = __fsqrt_rn(__fsub_rn(1.0f, rr));
      float d[3];
#pragma unroll
      for (int k2 = 0; k2 < 3; k2++)
        d[k2] = __fadd_rn(__fadd_rn(__fmul_rn(x, tx[k2]), __fmul_rn(y, ty[k2])), __fmul_rn(z, n[k2]));
      fnorm(d);
      const uint64_t w = slot * perHit + sIdx;
      if (w >= capacity)
      {
        atomicOr(errorWord, kErrLayout);
        break;
      }
      out[2 * w + 0] = make_float4(o[0], o[1], o[2], 0.0f);
      out[2 * w + 1] = make_float4(d[0], d[1], d[2], length);
      if (owner) owner[w] = (uint32_t)i;
    }
  }
}

uint32_t grid_for(uint64_t n, int numSMs)
{
  uint64_t g = (n + kThreads - 1) / kThreads;
  const uint64_t cap = (uint64_t)numSMs * 16;
  return (uint32_t)(g < 1 ? 1 : (g > cap ? cap : g));
}

void host_cross(const double a[3], const double b[3], double o[3])
{
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

void host_norm(double v[3])
{
  const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= l;
  v[1] /= l;
  v[2] /= l;
}

}  // namespace

extern "C" {

int hrt_gen_eye_rays(hrt_context* ctx, const float projInv[16], const float worldViewInv[16], uint32_t width,
                     uint32_t height, float tNear, float tFar, float* rays, void* stream)
{
  if (!ctx || !projInv || !worldViewInv || (!rays && width && height)) return HRT_ERR_INVALID_ARGUMENT;
  if (!aligned_to(rays, 16)) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "ray array must be 16-byte aligned");
  if ((uint64_t)width * height == 0) return HRT_OK;
  cudaSetDevice(ctx->device);
  Mat4 p, v;
  std::memcpy(p.m, projInv, sizeof(p.m));
  std::memcpy(v.m, worldViewInv, sizeof(v.m));
  k_eye_rays<<<grid_for((uint64_t)width * height, ctx->numSMs), kThreads, 0, (cudaStream_t)stream>>>(
      p, v, width, height, tNear, tFar, reinterpret_cast<float4*>(rays));
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? HRT_OK : cuda_fail(ctx, e, "k_eye_rays");
}

int hrt_gen_pinhole_rays(hrt_context* ctx, const float eye[3], const float target[3], const float up[3], float fovDeg,
                         uint32_t width, uint32_t height, float tmin, float tmax, float* rays, void* stream)
{
  if (!ctx || !eye || !target || !up || (!rays && width && height)) return HRT_ERR_INVALID_ARGUMENT;
  if (!aligned_to(rays, 16)) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "ray array must be 16-byte aligned");
  if ((uint64_t)width * height == 0) return HRT_OK;
  cudaSetDevice(ctx->device);
  // the frame, as the host generator sets it up (heavyrt_gb300/csrc/workload.c)
  double f[3] = {target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]};
  host_norm(f);
  const double u0[3] = {up[0], up[1], up[2]};
  double rgt[3], u[3];
  host_cross(f, u0, rgt);
  host_norm(rgt);
  host_cross(rgt, f, u);
  Pinhole c;
  for (int k = 0; k < 3; k++)
  {
    c.f[k] = (float)f[k];
    c.rgt[k] = (float)rgt[k];
    c.up[k] = (float)u[k];
  }
  c.th = (float)std::tan(0.5 * (double)fovDeg * 3.14159265358979323846 / 180.0);
  c.aspect = (float)((double)width / (double)height);
  std::memcpy(c.eye, eye, sizeof(c.eye));
  k_pinhole_rays<<<grid_for((uint64_t)width * height, ctx->numSMs), kThreads, 0, (cudaStream_t)stream>>>(
      c, width, height, tmin, tmax, reinterpret_cast<float4*>(rays));
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? HRT_OK : cuda_fail(ctx, e, "k_pinhole_rays");
}

int hrt_gen_ao_rays(hrt_scene* s, uint64_t seed, const float* eyeRays, const hrt_hit* hits, uint64_t nEye,
                    uint32_t perHit, float length, float offset, float* aoRays, uint32_t* owner, uint64_t capacity,
                    uint64_t* count, void* stream)
{
  if (!s || !count) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = s->ctx;
  *count = 0;
  if (!aligned_to(eyeRays, 16) || !aligned_to(hits, 16) || !aligned_to(aoRays, 16) || !aligned_to(owner, 4))
    return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "ray and hit arrays must be 16-byte aligned, owners 4-byte aligned");
  if (nEye == 0 || perHit == 0) return HRT_OK;
  if (!eyeRays || !hits || !aoRays) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "null ray, hit or output pointer");
  if (nEye > 0xFFFFFFFFull) return fail(ctx, HRT_ERR_CAPACITY, "more than 2^32-1 eye rays");
  std::lock_guard<std::mutex> lk(s->mu);
  for (const Instance& in : s->insts)
    if (!in.identity) return fail(ctx, HRT_ERR_UNSUPPORTED, "AO rays need identity instances (object = world space)");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<GeomPtr> hg(s->geoms.size());
  for (size_t i = 0; i < hg.size(); i++) hg[i] = GeomPtr{s->geoms[i].verts, s->geoms[i].sortedIdx, s->geoms[i].nTris};
  const uint32_t nBlocks = (uint32_t)((nEye + kThreads * 4 - 1) / (kThreads * 4));
  GeomPtr* dGeoms = nullptr;
  uint32_t* dBlock = nullptr;
  unsigned long long* dTotal = nullptr;
  uint32_t* dErr = nullptr;
  HRT_CUDA(ctx, cudaMallocAsync((void**)&dGeoms, sizeof(GeomPtr) * (hg.empty() ? 1 : hg.size()), st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&dBlock, sizeof(uint32_t) * nBlocks, st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&dTotal, sizeof(unsigned long long) + 2 * sizeof(uint32_t), st));
  dErr = reinterpret_cast<uint32_t*>(dTotal + 1);
  if (!hg.empty())
    HRT_CUDA(ctx, cudaMemcpyAsync(dGeoms, hg.data(), sizeof(GeomPtr) * hg.size(), cudaMemcpyHostToDevice, st));
  HRT_CUDA(ctx, cudaMemsetAsync(dErr, 0, sizeof(uint32_t), st));
  const float4* h4 = reinterpret_cast<const float4*>(hits);
  k_ao_count<<<nBlocks, kThreads, 0, st>>>(h4, nEye, dBlock);
  k_ao_scan<<<1, 1024, 0, st>>>(dBlock, nBlocks, dTotal);
  k_ao_emit<<<nBlocks, kThreads, 0, st>>>(seed, reinterpret_cast<const float4*>(eyeRays), h4, nEye, dGeoms,
                                          (uint32_t)hg.size(), dBlock, perHit, length, offset,
                                          reinterpret_cast<float4*>(aoRays), owner, capacity, dErr);
  HRT_CUDA(ctx, cudaGetLastError());
  unsigned long long total = 0;
  uint32_t err = 0;
  HRT_CUDA(ctx, cudaMemcpyAsync(&total, dTotal, sizeof(total), cudaMemcpyDeviceToHost, st));
  HRT_CUDA(ctx, cudaMemcpyAsync(&err, dErr, sizeof(err), cudaMemcpyDeviceToHost, st));
  HRT_CUDA(ctx, cudaFreeAsync(dGeoms, st));
  HRT_CUDA(ctx, cudaFreeAsync(dBlock, st));
  HRT_CUDA(ctx, cudaFreeAsync(dTotal, st));
  HRT_CUDA(ctx, cudaStreamSynchronize(st));
  *count = (uint64_t)total * perHit;
  if (err & kErrIndexRange) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "a hit names a geometry or triangle out of range");
  if (*count > capacity) return fail(ctx, HRT_ERR_CAPACITY, "AO output buffer too small");
  return HRT_OK;
}

}  // extern "C"
