// Drives the engine through HeavyRT's ISceneObject interface the way the
// eye-ray / RTAO renderers do: create through the factory function, add one
// geometry, instance it, commit, then call RayQuery_NearestHit and
// RayQuery_AnyHit once per ray from several host threads at once.
//
//   adapter_harness scene.bin rays.bin out_prefix threads layout [normals.bin params.bin]
// scene.bin: "HRTSCN01", u64 nVerts, u64 nIdx, float4 verts, u32 idx
// rays.bin:  "HRTRAY01", u64 n, 8 floats per ray
// writes out_prefix.hits (32 B per ray), out_prefix.any (1 B per ray) and
// prints the scene counts.  With normals.bin ("HRTNRM01", u64 n, float4
// normals) and params.bin (float projInv[16], worldViewInv[16], u32 width,
// height, float zNear, zFar, u32 raysPerPixel, float aoMaxRadius, power,
// normMatrix[16]) it also renders the example renderers' frames on the
// adapter's scene into host memory, as a renderer's Render() would:
// out_prefix.rtao and out_prefix.eye (uint32 colour per pixel).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <thread>
#include <vector>

#include "CrossRT.h"
#include "hrt.h"

ISceneObject* MakeGpuLBVHRT(const char* a_implName, const char* a_buildName, const char* a_layoutName);
hrt_scene*    GpuLBVHRT_Scene(ISceneObject* scene);
hrt_context*  GpuLBVHRT_Context(ISceneObject* scene);

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
  if (argc != 6 && argc != 8)
  {
    std::fprintf(stderr, "usage: %s scene.bin rays.bin out_prefix threads layout [normals.bin params.bin]\n", argv[0]);
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
  if (argc == 8)
  {
    std::vector<char> nb, pb;
    if (!read_file(argv[6], "HRTNRM01", nb) || std::ifstream(argv[7], std::ios::binary).fail()) return 3;
    std::ifstream pf(argv[7], std::ios::binary);
    pb.assign(std::istreambuf_iterator<char>(pf), std::istreambuf_iterator<char>());
    if (pb.size() != 220) return 3;
    uint64_t nN;
    std::memcpy(&nN, nb.data() + 8, 8);
    hrt_rtao_params p;
    uint32_t R;
    float normMatrix[16];
    std::memcpy(p.projInv, pb.data(), 64);
    std::memcpy(p.worldViewInv, pb.data() + 64, 64);
    std::memcpy(&p.width, pb.data() + 128, 4);
    std::memcpy(&p.height, pb.data() + 132, 4);
    std::memcpy(&p.zNear, pb.data() + 136, 4);
    std::memcpy(&p.zFar, pb.data() + 140, 4);
    std::memcpy(&R, pb.data() + 144, 4);
    std::memcpy(&p.aoMaxRadius, pb.data() + 148, 4);
    std::memcpy(&p.power, pb.data() + 152, 4);
    std::memcpy(normMatrix, pb.data() + 156, 64);
    hrt_frame* frame = nullptr;
    std::vector<float> tile(2 * (size_t)HRT_AO_TILE_SIZE * HRT_AO_TILE_SIZE * R);
    std::vector<uint32_t> rtao((size_t)p.width * p.height, 0xDEADBEEFu), eye(rtao.size(), 0xDEADBEEFu);
    int st = hrt_frame_create(GpuLBVHRT_Context(s), &frame);
    if (st == HRT_OK) st = hrt_rtao_qmc_tile(R, tile.data());
    if (st == HRT_OK) st = hrt_frame_set_ao_tile(frame, tile.data(), R);
    if (st == HRT_OK) st = hrt_frame_set_normals(frame, gid, reinterpret_cast<const float*>(nb.data() + 16), nN);
    if (st == HRT_OK) st = hrt_frame_render_rtao(frame, GpuLBVHRT_Scene(s), &p, normMatrix, rtao.data(), nullptr);
    if (st == HRT_OK)
      st = hrt_frame_render_eye(frame, GpuLBVHRT_Scene(s), p.projInv, p.worldViewInv, p.width, p.height, eye.data(),
                                nullptr);
    if (st != HRT_OK)
    {
      std::fprintf(stderr, "frame failed: %s\n", hrt_context_last_error(GpuLBVHRT_Context(s)));
      return 4;
    }
    hrt_frame_destroy(frame);
    std::ofstream(std::string(argv[3]) + ".rtao", std::ios::binary).write(reinterpret_cast<const char*>(rtao.data()),
                                                                        4 * rtao.size());
    std::ofstream(std::string(argv[3]) + ".eye", std::ios::binary).write(reinterpret_cast<const char*>(eye.data()),
                                                                       4 * eye.size());
  }
  const LiteMath::float4* boxes = s->GetGeomBoxes();
  std::printf("name=%s build=%s geoms=%u insts=%u gid=%u iid=%u box=%g,%g,%g,%g,%g,%g bvh_bytes=%zu\n", s->Name(),
              s->BuildName(), s->GetGeomNum(), s->GetInstNum(), gid, iid, boxes ? boxes[0].x : 0.0,
              boxes ? boxes[0].y : 0.0, boxes ? boxes[0].z : 0.0, boxes ? boxes[1].x : 0.0, boxes ? boxes[1].y : 0.0,
              boxes ? boxes[1].z : 0.0, s->GetStats().bvhTotalSize);
  DeleteSceneRT(s);
  return 0;
}

void DeleteSceneRT(ISceneObject* a_impl) { delete a_impl; }
