// Minimal vector types for building the ISceneObject adapter without HeavyRT's
// LiteMath (used by the engine's own adapter tests).  Only what the interface
// signatures need: float4 and a column-major float4x4 with the (row, col)
// accessor.  A real integration compiles the adapter against HeavyRT's
// core/CrossRT.h and its LiteMath instead of this directory.
#pragma once

namespace LiteMath
{

struct float4
{
  float x, y, z, w;
  float4() : x(0.0f), y(0.0f), z(0.0f), w(0.0f) {}
  float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  float&       operator[](int i) { return (&x)[i]; }
  const float& operator[](int i) const { return (&x)[i]; }
};

struct float4x4
{
  float4 m_col[4];  // column c holds M(0..3, c)
  float4x4()
  {
    for (int c = 0; c < 4; c++)
    {
      m_col[c] = float4();
      m_col[c][c] = 1.0f;
    }
  }
  float&       operator()(int r, int c) { return m_col[c][r]; }
  const float& operator()(int r, int c) const { return m_col[c][r]; }
};

}  // namespace LiteMath
