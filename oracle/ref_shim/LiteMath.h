// Minimal stand-in for the LiteMath vector library, written for this project.
//
// HeavyRT includes "LiteMath.h" from the git submodule external/LiteMath
// (msu-graphics-group/LiteMath), which is absent from the reference snapshot
// (the directory is empty and the pinned commit is unknown).  This header
// supplies only the names and signatures that the reference's LBVH builder and
// BVH2CommonRT traversal use, so that those reference sources compile unchanged
// as a CPU checker.  It is test infrastructure, never linked into the engine.
//
// Arithmetic choices (they define the checker, and the engine's kernels and the
// C restatement in oracle/ follow the same choices):
//   * every operation is a plain IEEE-754 binary32 operation, evaluated left to
//     right, with no fused multiply-add (the checker is compiled with
//     -ffp-contract=off);
//   * min(a,b) = (a < b) ? a : b and max(a,b) = (a > b) ? a : b, component-wise;
//   * dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z;
//   * cross(a,b) = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x);
//   * float4x4 is stored column-major; M*v sums the four column terms left to
//     right: ((c0*v.x + c1*v.y) + c2*v.z) + c3*v.w.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cfloat>
#include <limits>

#ifndef MAXFLOAT
#define MAXFLOAT FLT_MAX
#endif
#ifndef M_TWOPI
#define M_TWOPI 6.28318530717958647692f  // 2 pi as a float (the renderers' sample mapping)
#endif

namespace LiteMath
{
  typedef unsigned int uint;

  static inline float min(float a, float b) { return (a < b) ? a : b; }
  static inline float max(float a, float b) { return (a > b) ? a : b; }
  static inline int   min(int a, int b)     { return (a < b) ? a : b; }
  static inline int   max(int a, int b)     { return (a > b) ? a : b; }
  static inline uint  min(uint a, uint b)   { return (a < b) ? a : b; }
  static inline uint  max(uint a, uint b)   { return (a > b) ? a : b; }
  static inline float abs(float a)          { return std::fabs(a); }
  static inline float sign(float a)         { return (a > 0.0f) ? 1.0f : ((a < 0.0f) ? -1.0f : 0.0f); }
  static inline int   sign(int a)           { return (a > 0) ? 1 : ((a < 0) ? -1 : 0); }
  static inline float clamp(float x, float a, float b) { return min(max(x, a), b); }

  static inline int   as_int(float f)   { int r;   std::memcpy(&r, &f, 4); return r; }
  static inline uint  as_uint(float f)  { uint r;  std::memcpy(&r, &f, 4); return r; }
  static inline float as_float(int i)   { float r; std::memcpy(&r, &i, 4); return r; }
  static inline float as_float(uint i)  { float r; std::memcpy(&r, &i, 4); return r; }

  // ---------------------------------------------------------------- vectors
  template <typename T> struct vec2_t
  {
    T x, y;
    vec2_t() : x(0), y(0) {}
    explicit vec2_t(T a) : x(a), y(a) {}
    vec2_t(T a, T b) : x(a), y(b) {}
    T&       operator[](int i)       { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
  };

  template <typename T> struct vec3_t
  {
    T x, y, z;
    vec3_t() : x(0), y(0), z(0) {}
    explicit vec3_t(T a) : x(a), y(a), z(a) {}
    vec3_t(T a, T b, T c) : x(a), y(b), z(c) {}
    T&       operator[](int i)       { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
  };

  template <typename T> struct alignas(16) vec4_t
  {
    T x, y, z, w;
    vec4_t() : x(0), y(0), z(0), w(0) {}
    explicit vec4_t(T a) : x(a), y(a), z(a), w(a) {}
    vec4_t(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    // element-wise conversion, e.g. int4(float4) truncates each component
    template <typename U> explicit vec4_t(const vec4_t<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
    T&       operator[](int i)       { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
  };

  typedef vec2_t<float> float2;  typedef vec3_t<float> float3;  typedef vec4_t<float> float4;
  typedef vec2_t<int>   int2;    typedef vec3_t<int>   int3;    typedef vec4_t<int>   int4;
  typedef vec2_t<uint>  uint2;   typedef vec3_t<uint>  uint3;   typedef vec4_t<uint>  uint4;

  static_assert(sizeof(float3) == 12, "float3 must be 12 bytes (BVHNode is 32 bytes)");
  static_assert(sizeof(float4) == 16, "float4 must be 16 bytes");
  static_assert(sizeof(uint2)  == 8,  "uint2 must be 8 bytes");

#define HRT_SHIM_BINOP(OP)                                                                                          \
  template <typename T> static inline vec2_t<T> operator OP(vec2_t<T> a, vec2_t<T> b) { return vec2_t<T>(a.x OP b.x, a.y OP b.y); } \
  template <typename T> static inline vec3_t<T> operator OP(vec3_t<T> a, vec3_t<T> b) { return vec3_t<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z); } \
  template <typename T> static inline vec4_t<T> operator OP(vec4_t<T> a, vec4_t<T> b) { return vec4_t<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); } \
  template <typename T> static inline vec2_t<T> operator OP(vec2_t<T> a, T s) { return vec2_t<T>(a.x OP s, a.y OP s); } \
  template <typename T> static inline vec3_t<T> operator OP(vec3_t<T> a, T s) { return vec3_t<T>(a.x OP s, a.y OP s, a.z OP s); } \
  template <typename T> static inline vec4_t<T> operator OP(vec4_t<T> a, T s) { return vec4_t<T>(a.x OP s, a.y OP s, a.z OP s, a.w OP s); } \
  template <typename T> static inline vec2_t<T> operator OP(T s, vec2_t<T> a) { return vec2_t<T>(s OP a.x, s OP a.y); } \
  template <typename T> static inline vec3_t<T> operator OP(T s, vec3_t<T> a) { return vec3_t<T>(s OP a.x, s OP a.y, s OP a.z); } \
  template <typename T> static inline vec4_t<T> operator OP(T s, vec4_t<T> a) { return vec4_t<T>(s OP a.x, s OP a.y, s OP a.z, s OP a.w); }

  HRT_SHIM_BINOP(+)
  HRT_SHIM_BINOP(-)
  HRT_SHIM_BINOP(*)
  HRT_SHIM_BINOP(/)
#undef HRT_SHIM_BINOP

  template <typename T> static inline vec3_t<T> operator-(vec3_t<T> a) { return vec3_t<T>(-a.x, -a.y, -a.z); }
  template <typename T> static inline vec4_t<T> operator-(vec4_t<T> a) { return vec4_t<T>(-a.x, -a.y, -a.z, -a.w); }
  template <typename T> static inline vec3_t<T>& operator+=(vec3_t<T>& a, vec3_t<T> b) { a = a + b; return a; }
  template <typename T> static inline vec4_t<T>& operator+=(vec4_t<T>& a, vec4_t<T> b) { a = a + b; return a; }
  template <typename T> static inline vec3_t<T>& operator*=(vec3_t<T>& a, T s) { a = a * s; return a; }
  template <typename T> static inline vec4_t<T>& operator*=(vec4_t<T>& a, T s) { a = a * s; return a; }
  // component-wise division by a scalar (the renderers' `pos /= pos.w`)
  template <typename T> static inline vec3_t<T>& operator/=(vec3_t<T>& a, T s) { a = a / s; return a; }
  template <typename T> static inline vec4_t<T>& operator/=(vec4_t<T>& a, T s) { a = a / s; return a; }

  static inline float3 min(float3 a, float3 b) { return float3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
  static inline float3 max(float3 a, float3 b) { return float3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
  static inline float4 min(float4 a, float4 b) { return float4(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z), min(a.w, b.w)); }
  static inline float4 max(float4 a, float4 b) { return float4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)); }
  static inline float2 min(float2 a, float2 b) { return float2(min(a.x, b.x), min(a.y, b.y)); }
  static inline float2 max(float2 a, float2 b) { return float2(max(a.x, b.x), max(a.y, b.y)); }
  static inline float3 abs(float3 a) { return float3(abs(a.x), abs(a.y), abs(a.z)); }
  static inline float4 abs(float4 a) { return float4(abs(a.x), abs(a.y), abs(a.z), abs(a.w)); }
  static inline float3 sign(float3 a) { return float3(sign(a.x), sign(a.y), sign(a.z)); }
  static inline float4 clamp(float4 u, float a, float b) { return float4(clamp(u.x, a, b), clamp(u.y, a, b), clamp(u.z, a, b), clamp(u.w, a, b)); }
  // scalar given as any arithmetic type (the renderers' colour quantisation multiplies by an int)
  static inline float4 operator*(float4 a, float s) { return float4(a.x * s, a.y * s, a.z * s, a.w * s); }

  static inline float  dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
  static inline float  dot(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
  static inline float  dot3f(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
  static inline float3 cross(float3 a, float3 b) { return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
  static inline float  length(float3 a) { return std::sqrt(dot(a, a)); }
  static inline float  length3f(float4 a) { return std::sqrt(dot3f(a, a)); }
  static inline float3 normalize(float3 a) { return a * (1.0f / length(a)); }
  static inline float3 to_float3(float4 a) { return float3(a.x, a.y, a.z); }
  static inline float4 to_float4(float3 a, float w) { return float4(a.x, a.y, a.z, w); }
  static inline float  lerp(float a, float b, float t) { return a + t * (b - a); }

  // ---------------------------------------------------------------- matrix
  struct float4x4
  {
    float4 m_col[4]; // column-major: m_col[c][r] = M(r,c)
    float4x4() { identity(); }
    void identity()
    {
      for (int c = 0; c < 4; c++) { m_col[c] = float4(0.0f); m_col[c][c] = 1.0f; }
    }
    float&       operator()(int r, int c)       { return m_col[c][r]; }
    const float& operator()(int r, int c) const { return m_col[c][r]; }
    float4 get_col(int c) const { return m_col[c]; }
    void   set_col(int c, float4 v) { m_col[c] = v; }
  };

  static inline float4 operator*(const float4x4& m, float4 v)
  {
    float4 r;
    for (int i = 0; i < 4; i++)
      r[i] = ((m(i, 0) * v.x + m(i, 1) * v.y) + m(i, 2) * v.z) + m(i, 3) * v.w;
    return r;
  }

  static inline float4x4 operator*(const float4x4& a, const float4x4& b)
  {
    float4x4 r;
    for (int c = 0; c < 4; c++) r.m_col[c] = a * b.m_col[c];
    return r;
  }

  // Inverse through the adjugate: each entry of the inverse is a signed 3x3
  // minor of the transposed matrix divided by the determinant.
  static inline float4x4 inverse4x4(const float4x4& m)
  {
    float a[4][4];
    for (int r = 0; r < 4; r++)
      for (int c = 0; c < 4; c++) a[r][c] = m(r, c);
    auto minor3 = [&](int skipR, int skipC) {
      float s[3][3];
      int rr = 0;
      for (int r = 0; r < 4; r++)
      {
        if (r == skipR) continue;
        int cc = 0;
        for (int c = 0; c < 4; c++)
        {
          if (c == skipC) continue;
          s[rr][cc++] = a[r][c];
        }
        rr++;
      }
      return s[0][0] * (s[1][1] * s[2][2] - s[1][2] * s[2][1]) - s[0][1] * (s[1][0] * s[2][2] - s[1][2] * s[2][0]) +
             s[0][2] * (s[1][0] * s[2][1] - s[1][1] * s[2][0]);
    };
    float cof[4][4];
    for (int r = 0; r < 4; r++)
      for (int c = 0; c < 4; c++) cof[r][c] = (((r + c) & 1) ? -1.0f : 1.0f) * minor3(r, c);
    float det = a[0][0] * cof[0][0] + a[0][1] * cof[0][1] + a[0][2] * cof[0][2] + a[0][3] * cof[0][3];
    float4x4 inv;
    const float invDet = 1.0f / det;
    for (int r = 0; r < 4; r++)
      for (int c = 0; c < 4; c++) inv(r, c) = cof[c][r] * invDet;
    return inv;
  }

  // ---------------------------------------------------------------- boxes / rays
  struct Box4f
  {
    float4 boxMin;
    float4 boxMax;
    Box4f() : boxMin(+std::numeric_limits<float>::infinity()), boxMax(-std::numeric_limits<float>::infinity()) {}
    Box4f(float4 a, float4 b) : boxMin(a), boxMax(b) {}
    void include(const float4 p) { boxMin = min(boxMin, p); boxMax = max(boxMax, p); }
    void include(const Box4f& b) { boxMin = min(boxMin, b.boxMin); boxMax = max(boxMax, b.boxMax); }
    void intersect(const Box4f& b) { boxMin = max(boxMin, b.boxMin); boxMax = min(boxMax, b.boxMax); }
    float surfaceArea() const
    {
      const float4 e = boxMax - boxMin;
      return 2.0f * (e.x * e.y + e.x * e.z + e.y * e.z);
    }
    bool  axisAligned(int axis, float split) const { return boxMin[axis] == boxMax[axis] && boxMin[axis] == split; }
    float volume() const { const float4 e = boxMax - boxMin; return e.x * e.y * e.z; }
    float4 center() const { return (boxMin + boxMax) * 0.5f; }
    void  setStart(uint s) { boxMin.w = as_float(s); }
    void  setCount(uint c) { boxMax.w = as_float(c); }
    uint  getStart() const { return as_uint(boxMin.w); }
    uint  getCount() const { return as_uint(boxMax.w); }
  };

  static inline Box4f BoxBoxOverlap(const Box4f& a, const Box4f& b)
  {
    Box4f r = a;
    r.intersect(b);
    return r;
  }

  struct Ray4f
  {
    float4 posAndNear;
    float4 dirAndFar;
  };
}
