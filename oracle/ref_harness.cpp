// Checker harness around HeavyRT's own CPU code for the LBVH build and the
// BVH2CommonRT traversal.  Test infrastructure only: it is compiled from the
// reference sources by oracle/Makefile.ref into oracle/_ref/ and is never part
// of the engine.  It reads a scene / ray file, runs the reference's functions
// and writes their raw outputs so the tests can compare the C restatement
// (oracle/hrt_oracle.c) and the GPU engine against them.
//
// Reference entry points driven here:
//   LBVHBuilder::Reserve / stage kernels / BuildFromTriangles   core/builders/lbvh.cpp:84-139,228-319,732-827
//   BVH2CommonRT::AddGeom_Triangles3f (builder "cbvh_lbvh")     core/BVH2CommonRT_host.cpp:66-98
//   BVH2CommonRT::BVH2TraverseC32 (called directly, see below)  core/BVH2CommonRT.cpp:49-141
//
// Queries call BVH2TraverseC32 directly: with one instance, the reference's
// RayQuery_NearestHit gives the TLAS root-leaf a box distance of 1e37
// (core/BVH2CommonRT.cpp:146-150) and then skips the BLAS for every ray whose
// tFar is below 1e37 (:252).  Any-hit is derived as "nearest hit found",
// because BVH2CommonRT::RayQuery_AnyHit is a stub (core/BVH2CommonRT.cpp:281-292);
// the siblings define any-hit as the same traversal stopped at the first
// accepted triangle (core/BVH2CommonRTStacklessLBVH.cpp:161-165,235-240), which
// yields the same boolean.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "BVH2CommonRT.h"
#include "builders/cbvh_core.h"
#include "builders/cbvh_internal.h"
#include "builders/lbvh.h"

// ISceneObject::GetStats/ResetStats are defined out of line in the reference's
// FactoryRT.cpp, which would pull in every other implementation; these two
// definitions follow core/FactoryRT.cpp:82-104 so the vtable links.
MetricStats ISceneObject::GetStats()
{
  MetricStats stats = {};
  const double rays = double(m_stats.raysNumber) > 1.0 ? double(m_stats.raysNumber) : 1.0;
  stats.avgNC  = float(double(m_stats.NC) / rays);
  stats.avgLC  = float(double(m_stats.LC) / rays);
  stats.avgTC  = float(double(m_stats.TC) / rays);
  stats.avgBLB = float(double(m_stats.BLB) / rays);
  stats.avgSOC = float(double(m_stats.SOC) / rays);
  stats.avgSBL = float(double(m_stats.SBL) / rays);
  stats.bvhTotalSize  = m_stats.bvhTotalSize;
  stats.geomTotalSize = m_stats.geomTotalSize;
  return stats;
}
void ISceneObject::ResetStats() { m_stats.clear(); }

// Builders that the "cbvh_lbvh" path never reaches; the Embree archives and the
// SAH/ESC sources are not part of this checker.
namespace cbvh_embree
{
  cbvh::BVHTree BuildBVH(const float4*, size_t, const uint*, size_t, cbvh::BVHPresets)
  {
    std::fprintf(stderr, "ref_harness: Embree builder is not part of the checker\n");
    std::abort();
  }
}
namespace cbvh_internal
{
  cbvh::BVHTree BuildBVH4(const float4*, size_t, const uint*, size_t, BVHSettings)
  {
    std::fprintf(stderr, "ref_harness: SAH builder is not part of the checker\n");
    std::abort();
  }
  cbvh::BVHTree BuildBVH4(const Box4f*, size_t, const uint*, size_t, BVHSettings, OriginalInput)
  {
    std::fprintf(stderr, "ref_harness: SAH builder is not part of the checker\n");
    std::abort();
  }
}

namespace
{
  // Exposes the reference's protected traversal counters (core/CrossRT.h:170-191).
  struct RefRT : public BVH2CommonRT
  {
    explicit RefRT(const char* builder) : BVH2CommonRT(builder) {}
    const MetricsI& Counters() const { return m_stats; }
  };

  struct Scene
  {
    std::vector<float4>   verts;
    std::vector<uint32_t> idx;
  };

  bool ReadScene(const char* path, Scene& s)
  {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    char magic[8];
    uint64_t nv = 0, ni = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "HRTSCN01", 8) == 0 &&
              std::fread(&nv, 8, 1, f) == 1 && std::fread(&ni, 8, 1, f) == 1;
    if (ok)
    {
      s.verts.resize(nv);
      s.idx.resize(ni);
      ok = std::fread(s.verts.data(), 16, nv, f) == nv && std::fread(s.idx.data(), 4, ni, f) == ni;
    }
    std::fclose(f);
    return ok;
  }

  bool ReadRays(const char* path, std::vector<float4>& rays)
  {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    char magic[8];
    uint64_t n = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "HRTRAY01", 8) == 0 && std::fread(&n, 8, 1, f) == 1;
    if (ok)
    {
      rays.resize(2 * n);
      ok = std::fread(rays.data(), 16, 2 * n, f) == 2 * n;
    }
    std::fclose(f);
    return ok;
  }

  template <typename T> void Dump(const std::string& path, const T* data, size_t count)
  {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::fprintf(stderr, "cannot write %s\n", path.c_str()); std::exit(2); }
    if (count) std::fwrite(data, sizeof(T), count, f);
    std::fclose(f);
  }

  double NowMs()
  {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
  }

  // Stage outputs of the LBVH builder, in the order lbvh.cpp:745-767 calls them.
  void DumpStages(const Scene& s, const std::string& out)
  {
    const uint32_t nTris = uint32_t(s.idx.size() / 3);
    LBVHBuilder b;
    b.Reserve(nTris, cbvh2::BVH2_LEFT_OFFSET);
    const uint32_t ext = uint32_t(LBVHBuilder::powerOfTwo(nTris));
    b.kernel1D_RedunctionFromVertices(s.verts.data(), uint32_t(s.verts.size()));
    b.kernel1D_EvalMortonCodesFromTriangles(s.verts.data(), uint32_t(s.verts.size()), s.idx.data(), nTris, ext,
                                            b.runCodesAndIndices.data());
    float box[12] = {b.bboxMin.x, b.bboxMin.y, b.bboxMin.z, b.bboxMin.w, b.bboxMax.x, b.bboxMax.y,
                     b.bboxMax.z, b.bboxMax.w, b.zIndexScale.x, b.zIndexScale.y, b.zIndexScale.z, b.zIndexScale.w};
    Dump(out + ".bbox", box, 12);
    Dump(out + ".codes_unsorted", b.runCodesAndIndices.data(), nTris);
    std::sort(b.runCodesAndIndices.begin(), b.runCodesAndIndices.end(), [](uint2 x, uint2 y) { return x.x < y.x; });
    Dump(out + ".codes_sorted", b.runCodesAndIndices.data(), nTris);
    b.kernel1D_AppendInit(b.runCodesAndIndices.data(), nTris, b.codesEq.data(), b.prefixCodeEq.data());
    std::exclusive_scan(b.prefixCodeEq.begin(), b.prefixCodeEq.end(), b.prefixCodeEq.begin(), 0);
    b.kernel1D_AppendComplete(b.codesEq.data(), b.prefixCodeEq.data(), nTris);
    Dump(out + ".compressed", b.compressedCodes.data(), b.compressedCodes.size());
    Dump(out + ".runstarts", b.newIndices.data(), b.newIndices.size());

    // Whole build through the builder, to read the Karras + refit tree (LR
    // format, kept in m_tempNodes) and the peach relayout it produces.
    LBVHBuilder full;
    const size_t reserved = full.Reserve(nTris, cbvh2::BVH2_LEFT_OFFSET);
    std::vector<BVHNode>  nodes(reserved);
    std::vector<uint32_t> outIdx(nTris);
    full.BuildFromTriangles(s.verts.data(), uint32_t(s.verts.size()), s.idx.data(), uint32_t(s.idx.size()), nodes.data(),
                            uint32_t(reserved), outIdx.data());
    const size_t nLR = full.GetNodesNumber();
    Dump(out + ".lr_nodes", full.m_tempNodes.data(), nLR);
    Dump(out + ".lr_count", full.m_tempCount.data(), nLR);
    Dump(out + ".leaf_indices", outIdx.data(), outIdx.size());
    std::printf("{\"tris\": %u, \"leaves\": %d, \"reserved\": %zu}\n", nTris, full.m_leafNumber, reserved);
  }
}

int main(int argc, char** argv)
{
  if (argc < 4)
  {
    std::fprintf(stderr, "usage: %s stages|build|trace scene.bin out_prefix [rays.bin] [threads]\n", argv[0]);
    return 2;
  }
  const std::string cmd = argv[1];
  Scene s;
  if (!ReadScene(argv[2], s)) { std::fprintf(stderr, "cannot read scene %s\n", argv[2]); return 2; }
  const std::string out = argv[3];

  if (cmd == "stages")
  {
    DumpStages(s, out);
    return 0;
  }

  RefRT rt("cbvh_lbvh");
  rt.ClearGeom();
  const double t0 = NowMs();
  rt.AddGeom_Triangles3f((const float*)s.verts.data(), s.verts.size(), s.idx.data(), s.idx.size(), BUILD_LOW, 16);
  const double buildMs = NowMs() - t0;

  if (cmd == "build")
  {
    Dump(out + ".peach_nodes", rt.m_allNodes.data(), rt.m_allNodes.size());
    Dump(out + ".prim_indices", rt.m_primIndices.data(), rt.m_primIndices.size());
    Dump(out + ".indices_sorted", rt.m_indices.data(), rt.m_indices.size());
    std::printf("{\"build_ms\": %.3f, \"nodes\": %zu}\n", buildMs, rt.m_allNodes.size());
    return 0;
  }

  if (cmd == "trace" && argc >= 5)
  {
    std::vector<float4> rays;
    if (!ReadRays(argv[4], rays)) { std::fprintf(stderr, "cannot read rays %s\n", argv[4]); return 2; }
    const int64_t n = int64_t(rays.size() / 2);
    int threads = 1;
#ifdef _OPENMP
    threads = (argc >= 6) ? std::atoi(argv[5]) : omp_get_max_threads();
    if (threads < 1) threads = 1;
#endif
    std::vector<CRT_Hit> hits(n);
    std::vector<uint8_t> any(n);
    rt.ResetStats();
    const double t1 = NowMs();
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads)
#endif
    for (int64_t i = 0; i < n; i++)
    {
      const float4 pos = rays[2 * i + 0];
      const float4 dir = rays[2 * i + 1];
      uint32_t stack[STACK_SIZE];
      CRT_Hit hit;
      hit.t      = dir.w;
      hit.primId = uint32_t(-1);
      hit.instId = uint32_t(-1);
      hit.geomId = uint32_t(-1);
      hit.coords[0] = hit.coords[1] = hit.coords[2] = hit.coords[3] = 0.0f;
      rt.BVH2TraverseC32(to_float3(pos), to_float3(dir), pos.w, 0, 0, stack, &hit);
      hits[i] = hit;
      any[i]  = (hit.geomId != uint32_t(-1)) ? 1 : 0;
    }
    const double traceMs = NowMs() - t1;
    Dump(out + ".hits", hits.data(), hits.size());
    Dump(out + ".any", any.data(), any.size());
    std::printf("{\"build_ms\": %.3f, \"trace_ms\": %.3f, \"rays\": %lld, \"threads\": %d, \"avgNC\": %.4f, "
                "\"avgTC\": %.4f, \"avgBLB\": %.4f}\n",
                buildMs, traceMs, (long long)n, threads, n ? double(rt.Counters().NC) / double(n) : 0.0,
                n ? double(rt.Counters().TC) / double(n) : 0.0, n ? double(rt.Counters().BLB) / double(n) : 0.0);
    return 0;
  }
  std::fprintf(stderr, "unknown command %s\n", cmd.c_str());
  return 2;
}
