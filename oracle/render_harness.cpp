// Checker for the device frames of HeavyRT's two example renderers (TEST
// INFRASTRUCTURE ONLY).  The reference's own renderer kernels
// (examples/01_eye_rays/eye_ray.cpp, examples/02_rtao/rtao.cpp) and its
// quasi-random generator (core/common/qmc_sobol_niederreiter.cpp) are compiled
// unchanged against the LiteMath stand-in by oracle/Makefile.ref and driven
// here over one geometry traced by the reference's BVH2CommonRT.
//
//   render_harness qmc  raysPerPixel out_prefix
//       out.qmc  uint32[4][31]  the generator's direction table
//       out.tile float2[128*128*raysPerPixel]  RTAO's AO sample tile
//   render_harness eye  scene.bin params.bin out_prefix
//       out.packed uint32[W*H]  EyeRayCaster's packed pixel order (kernel_PackXY)
//       out.colors uint32[W*H]  the frame (kernel_InitEyeRay + kernel_RayTrace)
//   render_harness rtao scene.bin normals.bin params.bin out_prefix
//       out.eye_rays float4[2*W*H], out.eye_hits CRT_Hit[W*H],
//       out.positions float4[W*H] (kernel_TraceEyeRay2),
//       out.ao_rays float4[2*W*H*R] (kernel_InitAORay; zero where a pixel has no hit),
//       out.ao_hit uint8[W*H*R], out.visibility float[W*H], out.colors uint32[W*H]
//
// scene.bin: "HRTSCN01", u64 nVerts, u64 nIdx, float4 verts, u32 idx
// normals.bin: "HRTNRM01", u64 n, float4 normals
// params.bin: float projInv[16], float worldViewInv[16] (column-major),
//             u32 width, u32 height, float zNear, float zFar, u32 raysPerPixel,
//             float aoMaxRadius, float power, float normMatrix[16]
//
// Queries call BVH2TraverseC32 directly, as oracle/ref_harness.cpp does: with
// one instance the reference's RayQuery_NearestHit skips the geometry for
// every ray whose tFar is below 1e37 (core/BVH2CommonRT.cpp:146-150,252).
// For RTAO the hit's primId is mapped back to the original triangle: the
// renderer indexes its original index buffer with it (rtao.cpp:96-98) while
// BVH2CommonRT returns the position in sorted order (core/CrossRT.h:29).
// The eye-ray renderer colours by the returned primId as it stands.
//
// RTAO::InitQMCTable sits in rtao_host.cpp, which needs the scene loaders;
// its binning loop (rtao_host.cpp:383-414) is restated in QmcTile below over
// the reference's own initQuasirandomGenerator / rndQmcSobolN.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "BVH2CommonRT.h"
#include "builders/cbvh_core.h"
#include "builders/cbvh_internal.h"
#include "01_eye_rays/eye_ray.h"
#include "02_rtao/rtao.h"
#include "qmc_sobol_niederreiter.h"

// ISceneObject::GetStats/ResetStats live in the reference's FactoryRT.cpp,
// which would pull in every other implementation; the checker needs neither.
MetricStats ISceneObject::GetStats() { return MetricStats{}; }
void ISceneObject::ResetStats() { m_stats.clear(); }

namespace cbvh_embree
{
  cbvh::BVHTree BuildBVH(const float4*, size_t, const uint*, size_t, cbvh::BVHPresets)
  {
    std::fprintf(stderr, "render_harness: Embree builder is not part of the checker\n");
    std::abort();
  }
}
namespace cbvh_internal
{
  cbvh::BVHTree BuildBVH4(const float4*, size_t, const uint*, size_t, BVHSettings)
  {
    std::fprintf(stderr, "render_harness: SAH builder is not part of the checker\n");
    std::abort();
  }
  cbvh::BVHTree BuildBVH4(const Box4f*, size_t, const uint*, size_t, BVHSettings, OriginalInput)
  {
    std::fprintf(stderr, "render_harness: SAH builder is not part of the checker\n");
    std::abort();
  }
}

// The renderers' scene-loading and timing members live in eye_ray_host.cpp and
// rtao_host.cpp (scene loaders, glTF, Hydra XML); the checker sets the members
// directly, so these out-of-line members only have to exist for the vtables.
EyeRayCaster::EyeRayCaster() { m_pAccelStruct = nullptr; }
const char* EyeRayCaster::Name() const { return "EyeRayCaster"; }
bool EyeRayCaster::LoadScene(const char*) { return false; }
bool EyeRayCaster::LoadSingleMesh(const char*, const float*) { return false; }
void EyeRayCaster::Render(uint32_t*, uint32_t, uint32_t, const char*, int) {}
void EyeRayCaster::SetViewport(int, int, int, int) {}
void EyeRayCaster::GetExecutionTime(const char*, float a_out[4]) { a_out[0] = a_out[1] = a_out[2] = a_out[3] = 0.0f; }
CustomMetrics EyeRayCaster::GetMetrics() const { return CustomMetrics(); }
void EyeRayCaster::CastRaySingleBlock(uint32_t, uint32_t*, uint32_t) {}

RTAO::RTAO() {}
bool RTAO::LoadScene(const char*) { return false; }
bool RTAO::LoadSingleMesh(const char*, const float*) { return false; }
void RTAO::Render(uint32_t*, uint32_t, uint32_t, const char*, int) {}
void RTAO::SetViewport(int, int, int, int) {}
void RTAO::GetExecutionTime(const char*, float a_out[4]) { a_out[0] = a_out[1] = a_out[2] = a_out[3] = 0.0f; }
CustomMetrics RTAO::GetMetrics() const { return CustomMetrics(); }

namespace
{
  constexpr uint32_t kTile = 128;  // RTAO::AO_TILE_SIZE

  // BVH2CommonRT whose nearest-hit query runs the geometry's traversal directly.
  struct DirectRT : public BVH2CommonRT
  {
    DirectRT() : BVH2CommonRT("cbvh_lbvh") {}
    bool    originalPrimIds = false;
    CRT_Hit last{};

    CRT_Hit RayQuery_NearestHit(LiteMath::float4 posAndNear, LiteMath::float4 dirAndFar) override
    {
      uint32_t stack[STACK_SIZE];
      CRT_Hit hit;
      hit.t      = dirAndFar.w;
      hit.primId = uint32_t(-1);
      hit.instId = uint32_t(-1);
      hit.geomId = uint32_t(-1);
      hit.coords[0] = hit.coords[1] = hit.coords[2] = hit.coords[3] = 0.0f;
      BVH2TraverseC32(to_float3(posAndNear), to_float3(dirAndFar), posAndNear.w, 0, 0, stack, &hit);
      if (originalPrimIds && hit.primId != uint32_t(-1)) hit.primId = m_primIndices[hit.primId];
      last = hit;
      return hit;
    }
  };

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

  template <typename T> void Dump(const std::string& path, const T* data, size_t count)
  {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::fprintf(stderr, "cannot write %s\n", path.c_str()); std::exit(2); }
    if (count) std::fwrite(data, sizeof(T), count, f);
    std::fclose(f);
  }

  LiteMath::float4x4 ColMajor(const float* m)
  {
    LiteMath::float4x4 r;
    for (int c = 0; c < 4; c++)
      for (int k = 0; k < 4; k++) r(k, c) = m[4 * c + k];
    return r;
  }

  bool ReadScene(const char* path, std::vector<float4>& verts, std::vector<uint32_t>& idx)
  {
    const std::vector<char> b = Slurp(path);
    if (b.size() < 24 || std::memcmp(b.data(), "HRTSCN01", 8) != 0) return false;
    uint64_t nv, ni;
    std::memcpy(&nv, b.data() + 8, 8);
    std::memcpy(&ni, b.data() + 16, 8);
    if (b.size() != 24 + 16 * nv + 4 * ni) return false;
    verts.resize(nv);
    idx.resize(ni);
    std::memcpy(verts.data(), b.data() + 24, 16 * nv);
    std::memcpy(idx.data(), b.data() + 24 + 16 * nv, 4 * ni);
    return true;
  }

  // The AO sample tile as RTAO::InitQMCTable fills it (rtao_host.cpp:383-414):
  // point i of the 4-D sequence lands in the texel of its first two
  // coordinates, and the first raysPerPixel points of a texel keep their last two.
  void QmcTile(uint32_t raysPerPixel, std::vector<LiteMath::float2>& tile, unsigned int table[QRNG_DIMENSIONS][QRNG_RESOLUTION])
  {
    initQuasirandomGenerator(table);
    tile.assign(size_t(kTile) * kTile * raysPerPixel, LiteMath::float2());
    std::vector<uint32_t> filled(size_t(kTile) * kTile, 0);
    for (size_t i = 0; i < tile.size(); i++)
    {
      const float x = rndQmcSobolN(uint32_t(i), 0, table[0]);
      const float y = rndQmcSobolN(uint32_t(i), 1, table[0]);
      const float z = rndQmcSobolN(uint32_t(i), 2, table[0]);
      const float w = rndQmcSobolN(uint32_t(i), 3, table[0]);
      int ix = int(x * float(kTile));
      int iy = int(y * float(kTile));
      if (ix >= int(kTile)) ix = kTile - 1;
      if (iy >= int(kTile)) iy = kTile - 1;
      const uint32_t cell = uint32_t(iy) * kTile + uint32_t(ix);
      if (filled[cell] < raysPerPixel)
        tile[size_t(cell) * raysPerPixel + filled[cell]++] = LiteMath::float2(z, w);
    }
  }

  struct EyeProbe : public EyeRayCaster
  {
    void Run(const Params& p, std::shared_ptr<ISceneObject> rt, std::vector<uint32_t>& packed, std::vector<uint32_t>& colors)
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

  struct RtaoProbe : public RTAO
  {
    struct Out
    {
      std::vector<float4>   eyeRays, positions, aoRays;
      std::vector<CRT_Hit>  eyeHits;
      std::vector<uint8_t>  aoHit;
      std::vector<float>    visibility;
      std::vector<uint32_t> colors;
    };

    void Run(const Params& p, std::shared_ptr<DirectRT> rt, const std::vector<float4>& verts,
             const std::vector<uint32_t>& idx, const std::vector<float4>& normals, Out& o)
    {
      unsigned int table[QRNG_DIMENSIONS][QRNG_RESOLUTION];
      m_width = p.width;
      m_height = p.height;
      m_projInv = ColMajor(p.projInv);
      m_worldViewInv = ColMajor(p.worldViewInv);
      m_zNearFar = LiteMath::float2(p.zNear, p.zFar);
      m_aoMaxRadius = p.aoMaxRadius;
      m_power = p.power;
      m_aoRaysCount = p.raysPerPixel;
      m_normMatrices.assign(1, ColMajor(p.normMatrix));
      m_pAccelStruct = rt;
      m_matIdOffsets.assign(1, 0u);
      m_vertOffset.assign(1, 0u);
      m_triIndices = idx;
      m_vPos4f = verts;
      m_vNorm4f = normals;
      QmcTile(p.raysPerPixel, m_aoRandomsTile, table);

      const size_t nPix = size_t(p.width) * p.height, R = p.raysPerPixel;
      o.eyeRays.assign(2 * nPix, float4());
      o.eyeHits.assign(nPix, CRT_Hit{});
      o.positions.assign(nPix, float4());
      o.aoRays.assign(2 * nPix * R, float4());
      o.aoHit.assign(nPix * R, 0);
      o.visibility.assign(nPix, 0.0f);
      o.colors.assign(nPix, 0u);
      // RTAO::CalcAO (rtao.cpp:46-60) per pixel, row by row as CalcAOBlock
      // visits them, with each kernel's outputs recorded
      for (uint32_t j = 0; j < p.height; j++)
        for (uint32_t i = 0; i < p.width; i++)
        {
          const size_t pix = size_t(j) * p.width + i;
          float4 rayPosAndNear, rayDirAndFar, hitPosNorm;
          float  visibility;
          kernel_InitEyeRay(i, j, &rayPosAndNear, &rayDirAndFar, &visibility);
          o.eyeRays[2 * pix] = rayPosAndNear;
          o.eyeRays[2 * pix + 1] = rayDirAndFar;
          rt->originalPrimIds = true;
          kernel_TraceEyeRay2(i, j, &rayPosAndNear, &rayDirAndFar, &hitPosNorm);
          o.eyeHits[pix] = rt->last;
          o.positions[pix] = hitPosNorm;
          const bool hit = hitPosNorm.y < AO_HIT_BACK;
          for (uint32_t z = 0; z < m_aoRaysCount; z++)
          {
            kernel_InitAORay(i, j, z, &rayPosAndNear, &rayDirAndFar, &hitPosNorm);
            kernel_TraceAORay(i, j, &rayPosAndNear, &rayDirAndFar, &visibility);
            if (hit)
            {
              o.aoRays[2 * (pix * R + z)] = rayPosAndNear;
              o.aoRays[2 * (pix * R + z) + 1] = rayDirAndFar;
              o.aoHit[pix * R + z] = rt->last.geomId != uint32_t(-1) ? 1 : 0;
            }
          }
          o.visibility[pix] = visibility;
          kernel_AO2Color(i, j, &hitPosNorm, &visibility, o.colors.data());
        }
    }
  };

  bool ReadParams(const char* path, Params& p)
  {
    const std::vector<char> b = Slurp(path);
    if (b.size() != sizeof(Params)) return false;
    std::memcpy(&p, b.data(), sizeof(Params));
    return p.width > 0 && p.height > 0;
  }

  std::shared_ptr<DirectRT> Build(const std::vector<float4>& verts, const std::vector<uint32_t>& idx)
  {
    auto rt = std::make_shared<DirectRT>();
    rt->ClearGeom();
    rt->AddGeom_Triangles3f((const float*)verts.data(), verts.size(), idx.data(), idx.size(), BUILD_LOW, 16);
    return rt;
  }
}

int main(int argc, char** argv)
{
  const std::string cmd = argc > 1 ? argv[1] : "";
  if (cmd == "qmc" && argc == 4)
  {
    unsigned int table[QRNG_DIMENSIONS][QRNG_RESOLUTION];
    std::vector<LiteMath::float2> tile;
    QmcTile(uint32_t(std::atoi(argv[2])), tile, table);
    const std::string out = argv[3];
    Dump(out + ".qmc", &table[0][0], size_t(QRNG_DIMENSIONS) * QRNG_RESOLUTION);
    Dump(out + ".tile", tile.data(), tile.size());
    return 0;
  }
  if (cmd == "eye" && argc == 5)
  {
    std::vector<float4> verts;
    std::vector<uint32_t> idx;
    Params p;
    if (!ReadScene(argv[2], verts, idx) || !ReadParams(argv[3], p)) return 3;
    EyeProbe probe;
    std::vector<uint32_t> packed, colors;
    probe.Run(p, Build(verts, idx), packed, colors);
    const std::string out = argv[4];
    Dump(out + ".packed", packed.data(), packed.size());
    Dump(out + ".colors", colors.data(), colors.size());
    return 0;
  }
  if (cmd == "rtao" && argc == 6)
  {
    std::vector<float4> verts, normals;
    std::vector<uint32_t> idx;
    Params p;
    if (!ReadScene(argv[2], verts, idx) || !ReadParams(argv[4], p)) return 3;
    const std::vector<char> nb = Slurp(argv[3]);
    uint64_t nn = 0;
    if (nb.size() < 16 || std::memcmp(nb.data(), "HRTNRM01", 8) != 0) return 3;
    std::memcpy(&nn, nb.data() + 8, 8);
    if (nb.size() != 16 + 16 * nn || nn != verts.size()) return 3;
    normals.resize(nn);
    std::memcpy(normals.data(), nb.data() + 16, 16 * nn);
    RtaoProbe probe;
    RtaoProbe::Out o;
    probe.Run(p, Build(verts, idx), verts, idx, normals, o);
    const std::string out = argv[5];
    Dump(out + ".eye_rays", o.eyeRays.data(), o.eyeRays.size());
    Dump(out + ".eye_hits", o.eyeHits.data(), o.eyeHits.size());
    Dump(out + ".positions", o.positions.data(), o.positions.size());
    Dump(out + ".ao_rays", o.aoRays.data(), o.aoRays.size());
    Dump(out + ".ao_hit", o.aoHit.data(), o.aoHit.size());
    Dump(out + ".visibility", o.visibility.data(), o.visibility.size());
    Dump(out + ".colors", o.colors.data(), o.colors.size());
    return 0;
  }
  std::fprintf(stderr, "usage: %s qmc R out | eye scene params out | rtao scene normals params out\n", argv[0]);
  return 2;
}
