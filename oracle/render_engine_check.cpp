// HeavyRT's eye-ray renderer driving the GB300 engine (TEST INFRASTRUCTURE
// ONLY).  The renderer's own frame kernels (examples/01_eye_rays/eye_ray.cpp:
// kernel_PackXY through Clear(), kernel_InitEyeRay and kernel_RayTrace through
// CastRaySingle) are compiled unchanged by oracle/Makefile.ref and reach the
// engine only through their ISceneObject pointer, here the engine's adapter
// (heavyrt_gb300/csrc/scene_rt_adapter.cpp, MakeGpuLBVHRT), exactly as the
// renderer holds BVH2CommonRT in HeavyRT (eye_ray_host.cpp:297-342).
//
//   render_engine_check scene.bin params.bin out_prefix
//       out.packed uint32[W*H], out.colors uint32[W*H]
// (scene.bin / params.bin as for render_harness).  It needs a CUDA device: it
// is built wherever the reference sources are, and runs where that machine
// also has the GPU.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "CrossRT.h"
#include "01_eye_rays/eye_ray.h"

ISceneObject* MakeGpuLBVHRT(const char* a_implName, const char* a_buildName, const char* a_layoutName);

// ISceneObject::GetStats/ResetStats live in the reference's FactoryRT.cpp,
// which would pull in every other implementation.
MetricStats ISceneObject::GetStats() { return MetricStats{}; }
void ISceneObject::ResetStats() { m_stats.clear(); }

// The renderer's scene-loading and timing members (eye_ray_host.cpp) need the
// scene loaders; the check sets the members directly.
EyeRayCaster::EyeRayCaster() { m_pAccelStruct = nullptr; }
const char* EyeRayCaster::Name() const { return "EyeRayCaster"; }
bool EyeRayCaster::LoadScene(const char*) { return false; }
bool EyeRayCaster::LoadSingleMesh(const char*, const float*) { return false; }
void EyeRayCaster::Render(uint32_t*, uint32_t, uint32_t, const char*, int) {}
void EyeRayCaster::SetViewport(int, int, int, int) {}
void EyeRayCaster::GetExecutionTime(const char*, float a_out[4]) { a_out[0] = a_out[1] = a_out[2] = a_out[3] = 0.0f; }
CustomMetrics EyeRayCaster::GetMetrics() const { return CustomMetrics(); }
void EyeRayCaster::CastRaySingleBlock(uint32_t, uint32_t*, uint32_t) {}

namespace
{
  struct Params
  {
    float    projInv[16], worldViewInv[16];
    uint32_t width, height;
    float    zNear, zFar;
    uint32_t raysPerPixel;
    float    aoMaxRadius, power;
    float    normMatrix[16];
  };
  static_assert(sizeof(Params) == 220, "params.bin layout");

  std::vector<char> Slurp(const char* path)
  {
    std::vector<char> out;
    FILE* f = std::fopen(path, "rb");
    if (!f) return out;
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
    std::fclose(f);
    return out;
  }

  void Dump(const std::string& path, const uint32_t* data, size_t count)
  {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) std::exit(2);
    if (count) std::fwrite(data, sizeof(uint32_t), count, f);
    std::fclose(f);
  }

  LiteMath::float4x4 ColMajor(const float* m)
  {
    LiteMath::float4x4 r;
    for (int c = 0; c < 4; c++)
      for (int k = 0; k < 4; k++) r(k, c) = m[4 * c + k];
    return r;
  }

  struct EyeProbe : public EyeRayCaster
  {
    void Run(const Params& p, std::shared_ptr<ISceneObject> rt, std::vector<uint32_t>& packed,
             std::vector<uint32_t>& colors)
    {
      m_width = p.width;
      m_height = p.height;
      m_projInv = ColMajor(p.projInv);
      m_worldViewInv = ColMajor(p.worldViewInv);
      m_measureOverhead = 0;
      m_pAccelStruct = rt;
      m_packedXY.assign(size_t(p.width) * p.height, 0u);
      Clear(p.width, p.height, "color");  // PackXYBlock -> kernel_PackXY
      colors.assign(size_t(p.width) * p.height, 0u);
      for (uint32_t i = 0; i < p.width * p.height; i++) CastRaySingle(i, colors.data());
      packed = m_packedXY;
    }
  };
}

int main(int argc, char** argv)
{
  if (argc != 4)
  {
    std::fprintf(stderr, "usage: %s scene.bin params.bin out_prefix\n", argv[0]);
    return 2;
  }
  const std::vector<char> b = Slurp(argv[1]);
  uint64_t nv = 0, ni = 0;
  if (b.size() < 24 || std::memcmp(b.data(), "HRTSCN01", 8) != 0) return 3;
  std::memcpy(&nv, b.data() + 8, 8);
  std::memcpy(&ni, b.data() + 16, 8);
  if (b.size() != 24 + 16 * nv + 4 * ni) return 3;
  const std::vector<char> pb = Slurp(argv[2]);
  Params p;
  if (pb.size() != sizeof(Params)) return 3;
  std::memcpy(&p, pb.data(), sizeof(Params));
  std::shared_ptr<ISceneObject> rt(MakeGpuLBVHRT("GB300_LBVH", "cbvh_lbvh", ""));
  rt->ClearGeom();
  const uint32_t g = rt->AddGeom_Triangles3f(reinterpret_cast<const float*>(b.data() + 24), nv,
                                             reinterpret_cast<const uint32_t*>(b.data() + 24 + 16 * nv), ni,
                                             BUILD_HIGH, 16);
  rt->ClearScene();
  LiteMath::float4x4 id;
  rt->AddInstance(g, id);
  rt->CommitScene();
  EyeProbe probe;
  std::vector<uint32_t> packed, colors;
  probe.Run(p, rt, packed, colors);
  const std::string out = argv[3];
  Dump(out + ".packed", packed.data(), packed.size());
  Dump(out + ".colors", colors.data(), colors.size());
  return 0;
}
