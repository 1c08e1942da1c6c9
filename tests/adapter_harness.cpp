// Drives the engine through HeavyRT's ISceneObject interface the way the
// eye-ray / RTAO renderers do: create through the factory function, add one
// geometry, instance it, commit, then call RayQuery_NearestHit and
// RayQuery_AnyHit once per ray from several host threads at once.
//
//   adapter_harness scene.bin rays.bin out_prefix threads layout
// scene.bin: "HRTSCN01", u64 nVerts, u64 nIdx, float4 verts, u32 idx
// rays.bin:  "HRTRAY01", u64 n, 8 floats per ray
// writes out_prefix.hits (32 B per ray), out_prefix.any (1 B per ray) and
// prints the scene counts.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <thread>
#include <vector>

#include "CrossRT.h"

ISceneObject* MakeGpuLBVHRT(const char* a_implName, const char* a_buildName, const char* a_layoutName);

// Defined out of line by HeavyRT's factory translation unit (core/FactoryRT.cpp:82-104);
// this harness links no HeavyRT code, so it provides them.
MetricStats ISceneObject::GetStats() { return MetricStats{}; }
void ISceneObject::ResetStats() { m_stats.clear(); }

static bool read_file(const char* path, const char* magic, std::vector<char>& out)
{
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return out.size() >= 8 && std::memcmp(out.data(), magic, 8) == 0;
}

int main(int argc, char** argv)
{
  if (argc != 6)
  {
    std::fprintf(stderr, "usage: %s scene.bin rays.bin out_prefix threads layout\n", argv[0]);
    return 2;
  }
  std::vector<char> sc, ry;
  if (!read_file(argv[1], "HRTSCN01", sc) || !read_file(argv[2], "HRTRAY01", ry)) return 3;
  uint64_t nV, nI, nR;
  std::memcpy(&nV, sc.data() + 8, 8);
  std::memcpy(&nI, sc.data() + 16, 8);
  std::memcpy(&nR, ry.data() + 8, 8);
  const float* verts = reinterpret_cast<const float*>(sc.data() + 24);
  const uint32_t* idx = reinterpret_cast<const uint32_t*>(sc.data() + 24 + 16 * nV);
  const float* rays = reinterpret_cast<const float*>(ry.data() + 16);
  const int threads = std::atoi(argv[4]);

  ISceneObject* s = MakeGpuLBVHRT("GB300_LBVH", "cbvh_lbvh", argv[5]);
  s->ClearGeom();
  const uint32_t gid = s->AddGeom_Triangles3f(verts, nV, idx, nI, BUILD_HIGH, 16);
  LiteMath::float4x4 identity;
  s->ClearScene();
  const uint32_t iid = s->AddInstance(gid, identity);
  s->CommitScene(BUILD_MEDIUM);

  std::vector<CRT_Hit> hits(nR);
  std::vector<uint8_t> any(nR);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++)
    pool.emplace_back([&, t]() {
      for (uint64_t i = t; i < nR; i += threads)
      {
        const float* r = rays + 8 * i;
        const LiteMath::float4 p(r[0], r[1], r[2], r[3]), d(r[4], r[5], r[6], r[7]);
        hits[i] = s->RayQuery_NearestHit(p, d);
        any[i] = s->RayQuery_AnyHit(p, d) ? 1 : 0;
      }
    });
  for (auto& th : pool) th.join();

  const std::string prefix = argv[3];
  std::ofstream(prefix + ".hits", std::ios::binary).write(reinterpret_cast<const char*>(hits.data()), 32 * nR);
  std::ofstream(prefix + ".any", std::ios::binary).write(reinterpret_cast<const char*>(any.data()), nR);
  const LiteMath::float4* boxes = s->GetGeomBoxes();
  std::printf("name=%s build=%s geoms=%u insts=%u gid=%u iid=%u box=%g,%g,%g,%g,%g,%g bvh_bytes=%zu\n", s->Name(),
              s->BuildName(), s->GetGeomNum(), s->GetInstNum(), gid, iid, boxes ? boxes[0].x : 0.0,
              boxes ? boxes[0].y : 0.0, boxes ? boxes[0].z : 0.0, boxes ? boxes[1].x : 0.0, boxes ? boxes[1].y : 0.0,
              boxes ? boxes[1].z : 0.0, s->GetStats().bvhTotalSize);
  DeleteSceneRT(s);
  return 0;
}

void DeleteSceneRT(ISceneObject* a_impl) { delete a_impl; }
