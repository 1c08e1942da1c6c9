// Device arithmetic shared by the ray generators (raygen.cu) and the renderer
// frames (render.cu): the renderers' eye-ray set-up, RTAO::kernel_InitEyeRay
// (examples/02_rtao/rtao.cpp:133-144; examples/01_eye_rays/eye_ray.cpp:26-47)
// with EyeRayDirNormalized and transform_ray3f (examples/render_common.h:6-36).
// Every float operation is an explicit round-to-nearest intrinsic in the
// reference's order (mat x vec sums ((m0 x + m1 y) + m2 z) + m3 w, normalize(v)
// = v * (1 / sqrt(dot(v, v)))), so nothing is contracted into an FMA.
#pragma once

#include <cstdint>

namespace hrt
{
namespace rg
{

struct Mat4
{
  float m[16];  // column-major
};

__device__ __forceinline__ void mat_vec(const Mat4& M, const float v[4], float o[4])
{
  const float* m = M.m;
#pragma unroll
  for (int r = 0; r < 4; r++)
    o[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[r], v[0]), __fmul_rn(m[4 + r], v[1])), __fmul_rn(m[8 + r], v[2])),
                     __fmul_rn(m[12 + r], v[3]));
}

__device__ __forceinline__ float dot3(const float a[3], const float b[3])
{
  return __fadd_rn(__fadd_rn(__fmul_rn(a[0], b[0]), __fmul_rn(a[1], b[1])), __fmul_rn(a[2], b[2]));
}

__device__ __forceinline__ void normalize3(float v[3])
{
  const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot3(v, v)));
  v[0] = __fmul_rn(v[0], inv);
  v[1] = __fmul_rn(v[1], inv);
  v[2] = __fmul_rn(v[2], inv);
}

// The eye ray through the centre of pixel (x, y) of a width x height image.
__device__ __forceinline__ void eye_ray(const Mat4& projInv, const Mat4& worldViewInv, uint32_t x, uint32_t y,
                                        uint32_t width, uint32_t height, float tNear, float tFar, float4& posAndNear,
                                        float4& dirAndFar)
{
  const float fx = __fdiv_rn(__fadd_rn((float)x, 0.5f), (float)width);
  const float fy = __fdiv_rn(__fadd_rn((float)y, 0.5f), (float)height);
  const float pos[4] = {__fsub_rn(__fmul_rn(2.0f, fx), 1.0f), __fadd_rn(__fmul_rn(-2.0f, fy), 1.0f), 0.0f, 1.0f};
  float p[4];
  mat_vec(projInv, pos, p);
  float d[3] = {__fdiv_rn(p[0], p[3]), __fdiv_rn(p[1], p[3]), __fdiv_rn(p[2], p[3])};
  normalize3(d);
  const float o0[4] = {0.0f, 0.0f, 0.0f, 1.0f};
  const float o1[4] = {__fadd_rn(0.0f, __fmul_rn(100.0f, d[0])), __fadd_rn(0.0f, __fmul_rn(100.0f, d[1])),
                       __fadd_rn(0.0f, __fmul_rn(100.0f, d[2])), 1.0f};
  float a[4], b[4];
  mat_vec(worldViewInv, o0, a);
  mat_vec(worldViewInv, o1, b);
  float dir[3] = {__fsub_rn(b[0], a[0]), __fsub_rn(b[1], a[1]), __fsub_rn(b[2], a[2])};
  normalize3(dir);
  posAndNear = make_float4(a[0], a[1], a[2], tNear);
  dirAndFar = make_float4(dir[0], dir[1], dir[2], tFar);
}

}  // namespace rg
}  // namespace hrt
