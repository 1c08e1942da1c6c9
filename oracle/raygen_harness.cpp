// Checker for on-device ray generation (TEST INFRASTRUCTURE ONLY): the ray
// set-up of HeavyRT's renderers computed by the reference's own helpers
// (examples/render_common.h) compiled against the LiteMath stand-in.
//
//   raygen_harness eye params.bin out.bin
//     params: float projInv[16], float worldViewInv[16] (column-major),
//             uint32 width, uint32 height, float tNear, float tFar
//     out:    width*height rays {posAndNear, dirAndFar}, row-major pixels:
//             the body of RTAO::kernel_InitEyeRay (examples/02_rtao/rtao.cpp:133-144)
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <vector>

#include "render_common.h"

using namespace LiteMath;

static std::vector<char> slurp(const char* path)
{
  std::ifstream f(path, std::ios::binary);
  return std::vector<char>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

static float4x4 load_col_major(const float* m)
{
  float4x4 r;
  for (int c = 0; c < 4; c++)
    for (int k = 0; k < 4; k++) r(k, c) = m[4 * c + k];
  return r;
}

int main(int argc, char** argv)
{
  if (argc != 4) return 2;
  const std::vector<char> in = slurp(argv[2]);
  std::vector<float> out;
  if (std::strcmp(argv[1], "eye") == 0)
  {
    if (in.size() < 32 * 4 + 16) return 3;
    const float* m = reinterpret_cast<const float*>(in.data());
    uint32_t wh[2];
    float nf[2];
    std::memcpy(wh, in.data() + 128, 8);
    std::memcpy(nf, in.data() + 136, 8);
    const float4x4 projInv = load_col_major(m), worldViewInv = load_col_major(m + 16);
    out.resize(8 * (size_t)wh[0] * wh[1]);
    for (uint32_t y = 0; y < wh[1]; y++)
      for (uint32_t x = 0; x < wh[0]; x++)
      {
        float3 rayDir = EyeRayDirNormalized((float(x) + 0.5f) / float(wh[0]), (float(y) + 0.5f) / float(wh[1]), projInv);
        float3 rayPos = float3(0, 0, 0);
        transform_ray3f(worldViewInv, &rayPos, &rayDir);
        float* o = &out[8 * ((size_t)y * wh[0] + x)];
        o[0] = rayPos.x; o[1] = rayPos.y; o[2] = rayPos.z; o[3] = nf[0];
        o[4] = rayDir.x; o[5] = rayDir.y; o[6] = rayDir.z; o[7] = nf[1];
      }
  }
  else
    return 2;
  std::ofstream(argv[3], std::ios::binary).write(reinterpret_cast<const char*>(out.data()), 4 * out.size());
  return 0;
}
