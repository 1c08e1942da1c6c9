// GpuLBVHRT: HeavyRT's ISceneObject (core/CrossRT.h:64-193) implemented on the
// engine's C ABI (include/hrt.h), so that the eye-ray and RTAO renderers drive
// the GB300 engine through their unchanged ISceneObject pointer.
//
// Build with HeavyRT's core/ (CrossRT.h + LiteMath) first on the include
// path and register the factory in its CreateSceneRT (core/FactoryRT.cpp:29-78):
//   else if (className.find("GB300") != std::string::npos)
//     return MakeGpuLBVHRT(a_implName, a_buildName, a_layoutName);
//
// Behaviour (same as the reference's BVH2CommonRT where it defines one):
//   * geometry and instances are copied at the call (core/BVH2CommonRT_host.cpp:66-164);
//   * RayQuery_* may be called concurrently from many host threads, as the
//     renderers do from OpenMP loops: concurrent calls are combined into one
//     batched GPU query (the first waiting thread traces everything queued,
//     the others wait for their slot), so a frame costs a few hundred
//     launches instead of one per ray;
//   * primId is the Morton-sorted position (REMAP_PRIM_ID off, core/CrossRT.h:29);
//   * errors have no channel in the interface (the reference prints and goes
//     on): failed calls log to stderr once per kind, return geometry/instance
//     id 0xFFFFFFFF and make queries report misses.
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "CrossRT.h"
#include "hrt.h"

namespace
{

constexpr uint32_t kNoId = 0xFFFFFFFFu;

int layout_from_name(const char* name)
{
  const std::string s = name ? name : "";
  if (s.find("Q8") != std::string::npos || s.find("q8") != std::string::npos) return HRT_LAYOUT_BVH4_Q8;
  if (s.find("16") != std::string::npos || s.find("Half") != std::string::npos || s.find("half") != std::string::npos)
    return HRT_LAYOUT_BVH4_F16;
  if (s.find("BVH4") != std::string::npos || s.find("bvh4") != std::string::npos) return HRT_LAYOUT_BVH4_F32;
  return HRT_LAYOUT_BVH2;
}

class GpuLBVHRT : public ISceneObject
{
public:
  GpuLBVHRT(const char* implName, const char* buildName, const char* layoutName)
      : m_impl(implName ? implName : "GB300_LBVH"), m_build(buildName ? buildName : "cbvh_lbvh")
  {
    const char* dev = std::getenv("HRT_DEVICE");
    int st = hrt_context_create(dev ? std::atoi(dev) : 0, &m_ctx);
    if (st == HRT_OK) st = hrt_scene_create(m_ctx, m_build.c_str(), &m_scene);
    if (st == HRT_OK && layoutName && *layoutName) st = hrt_scene_set_layout(m_scene, layout_from_name(layoutName));
    if (st != HRT_OK) report("create", st);
  }

  ~GpuLBVHRT() override
  {
    if (m_scene) hrt_scene_destroy(m_scene);
    if (m_stage) hrt_host_free(m_stage);
    if (m_ctx) hrt_context_destroy(m_ctx);
  }

  const char* Name() const override { return m_impl.c_str(); }
  const char* BuildName() const override { return m_build.c_str(); }

  void ClearGeom() override
  {
    if (!m_scene) return;
    check("ClearGeom", hrt_clear_geom(m_scene));
    m_boxes.clear();
  }

  uint32_t AddGeom_Triangles3f(const float* a_vpos3f, size_t a_vertNumber, const uint32_t* a_triIndices,
                               size_t a_indNumber, BuildQuality a_qualityLevel, size_t vByteStride) override
  {
    if (!m_scene) return kNoId;
    uint32_t id = kNoId;
    if (!check("AddGeom_Triangles3f", hrt_add_geom_triangles3f(m_scene, a_vpos3f, a_vertNumber, a_triIndices,
                                                               a_indNumber, (int)a_qualityLevel, vByteStride, &id)))
      return kNoId;
    refresh_boxes();
    return id;
  }

  void UpdateGeom_Triangles3f(uint32_t a_geomId, const float* a_vpos3f, size_t a_vertNumber,
                              const uint32_t* a_triIndices, size_t a_indNumber, BuildQuality a_qualityLevel,
                              size_t vByteStride) override
  {
    if (!m_scene) return;
    check("UpdateGeom_Triangles3f", hrt_update_geom_triangles3f(m_scene, a_geomId, a_vpos3f, a_vertNumber,
                                                                a_triIndices, a_indNumber, (int)a_qualityLevel,
                                                                vByteStride));
  }

  void ClearScene() override
  {
    if (m_scene) check("ClearScene", hrt_clear_scene(m_scene));
  }

  void CommitScene(BuildQuality a_qualityLevel) override
  {
    if (m_scene) check("CommitScene", hrt_commit_scene(m_scene, (int)a_qualityLevel));
  }

  uint32_t AddInstance(uint32_t a_geomId, const LiteMath::float4x4& a_matrix) override
  {
    if (!m_scene) return kNoId;
    float m[16];
    column_major(a_matrix, m);
    uint32_t id = kNoId;
    return check("AddInstance", hrt_add_instance(m_scene, a_geomId, m, &id)) ? id : kNoId;
  }

  void UpdateInstance(uint32_t a_instanceId, const LiteMath::float4x4& a_matrix) override
  {
    if (!m_scene) return;
    float m[16];
    column_major(a_matrix, m);
    check("UpdateInstance", hrt_update_instance(m_scene, a_instanceId, m));
  }

  CRT_Hit RayQuery_NearestHit(LiteMath::float4 posAndNear, LiteMath::float4 dirAndFar) override
  {
    Request r(0, posAndNear, dirAndFar);
    submit(&r);
    return r.hit;
  }

  bool RayQuery_AnyHit(LiteMath::float4 posAndNear, LiteMath::float4 dirAndFar) override
  {
    Request r(1, posAndNear, dirAndFar);
    submit(&r);
    return r.any != 0;
  }

  MetricStats GetStats() override
  {
    MetricStats st = {};
    uint32_t n = 0;
    if (m_scene && hrt_get_geom_num(m_scene, &n) == HRT_OK)
      for (uint32_t g = 0; g < n; g++)
      {
        uint64_t info[4] = {0, 0, 0, 0};
        if (hrt_geom_info(m_scene, g, info, nullptr) == HRT_OK) st.bvhTotalSize += info[3];
      }
    return st;
  }

  void ResetStats() override {}

  uint32_t GetGeomNum() const override
  {
    uint32_t n = 0;
    if (m_scene) hrt_get_geom_num(m_scene, &n);
    return n;
  }

  uint32_t GetInstNum() const override
  {
    uint32_t n = 0;
    if (m_scene) hrt_get_inst_num(m_scene, &n);
    return n;
  }

  const LiteMath::float4* GetGeomBoxes() const override
  {
    return m_boxes.empty() ? nullptr : m_boxes.data();
  }

  hrt_scene*   Scene() const { return m_scene; }
  hrt_context* Context() const { return m_ctx; }

  // Batched queries for callers that hold whole ray arrays (one GPU call).
  void RayQuery_NearestHitBatch(const LiteMath::float4* posAndNear, const LiteMath::float4* dirAndFar, size_t n,
                                CRT_Hit* out)
  {
    std::vector<float> rays(8 * n);
    for (size_t i = 0; i < n; i++) pack(posAndNear[i], dirAndFar[i], &rays[8 * i]);
    std::vector<hrt_hit> h(n);
    if (!m_scene || !check("RayQuery_NearestHitBatch", hrt_query_nearest_host(m_scene, rays.data(), n, h.data())))
      for (size_t i = 0; i < n; i++) out[i] = miss(dirAndFar[i].w);
    else
      for (size_t i = 0; i < n; i++) std::memcpy(&out[i], &h[i], sizeof(CRT_Hit));
  }

private:
  struct Request
  {
    int     kind;
    float   ray[8];
    CRT_Hit hit;
    uint8_t any = 0;
    bool    done = false;
    Request(int k, const LiteMath::float4& p, const LiteMath::float4& d) : kind(k) { pack(p, d, ray); }
  };

  static void pack(const LiteMath::float4& p, const LiteMath::float4& d, float* r)
  {
    r[0] = p.x; r[1] = p.y; r[2] = p.z; r[3] = p.w;
    r[4] = d.x; r[5] = d.y; r[6] = d.z; r[7] = d.w;
  }

  static CRT_Hit miss(float tFar)
  {
    CRT_Hit h;
    h.t = tFar;
    h.primId = h.instId = h.geomId = kNoId;
    h.coords[0] = h.coords[1] = h.coords[2] = h.coords[3] = 0.0f;
    return h;
  }

  static void column_major(const LiteMath::float4x4& a, float* m)
  {
    for (int c = 0; c < 4; c++)
      for (int r = 0; r < 4; r++) m[4 * c + r] = a(r, c);
  }

  // Flat combining: every caller queues its request; a caller that finds no
  // batch in flight takes the whole queue, traces it with one query per kind
  // and wakes the others; callers whose request is still queued then repeat.
  void submit(Request* r)
  {
    std::unique_lock<std::mutex> lk(m_qmu);
    m_queue.push_back(r);
    while (!r->done)
    {
      if (m_busy)
      {
        m_qcv.wait(lk);
        continue;
      }
      m_busy = true;
      std::vector<Request*> batch;
      batch.swap(m_queue);
      lk.unlock();
      run(batch);
      lk.lock();
      for (Request* q : batch) q->done = true;
      m_busy = false;
      m_qcv.notify_all();
    }
  }

  void run(const std::vector<Request*>& batch)
  {
    for (int kind = 0; kind < 2; kind++)
    {
      size_t n = 0;
      for (const Request* q : batch) n += (q->kind == kind);
      if (n == 0) continue;
      const size_t need = 32 * n + (kind == 0 ? sizeof(hrt_hit) * n : n);
      if (need > m_stageBytes)
      {
        if (m_stage) hrt_host_free(m_stage);
        m_stage = nullptr;
        m_stageBytes = 0;
        if (hrt_host_alloc(2 * need, &m_stage) == HRT_OK) m_stageBytes = 2 * need;
      }
      float* rays = static_cast<float*>(m_stage);
      void* out = m_stage ? static_cast<char*>(m_stage) + 32 * n : nullptr;
      size_t k = 0;
      if (rays)
        for (const Request* q : batch)
          if (q->kind == kind) std::memcpy(rays + 8 * k++, q->ray, 32);
      const int st = !m_scene || !rays ? HRT_ERR_STATE
                     : kind == 0       ? hrt_query_nearest_host(m_scene, rays, n, static_cast<hrt_hit*>(out))
                                       : hrt_query_any_host(m_scene, rays, n, static_cast<uint8_t*>(out));
      const bool ok = check(kind == 0 ? "RayQuery_NearestHit" : "RayQuery_AnyHit", st);
      k = 0;
      for (Request* q : batch)
      {
        if (q->kind != kind) continue;
        if (kind == 0)
        {
          if (ok) std::memcpy(&q->hit, static_cast<const hrt_hit*>(out) + k, sizeof(CRT_Hit));
          else q->hit = miss(q->ray[7]);
        }
        else
          q->any = ok ? static_cast<const uint8_t*>(out)[k] : 0;
        k++;
      }
    }
  }

  void refresh_boxes()
  {
    const uint32_t n = GetGeomNum();
    m_boxes.assign(2 * (size_t)n, LiteMath::float4());
    if (n) hrt_get_geom_boxes(m_scene, reinterpret_cast<float*>(m_boxes.data()), n);
  }

  bool check(const char* what, int status)
  {
    if (status == HRT_OK) return true;
    report(what, status);
    return false;
  }

  void report(const char* what, int status)
  {
    std::lock_guard<std::mutex> g(m_logmu);
    if (m_reported.find(what) != std::string::npos) return;  // once per call kind
    m_reported += what;
    m_reported += ';';
    std::fprintf(stderr, "[GpuLBVHRT] %s failed: %s (%s)\n", what, hrt_status_string(status),
                 m_ctx ? hrt_context_last_error(m_ctx) : "no context");
  }

  std::string                   m_impl, m_build;
  hrt_context*                  m_ctx = nullptr;
  hrt_scene*                    m_scene = nullptr;
  std::vector<LiteMath::float4> m_boxes;  // boxMin, boxMax per geometry
  std::mutex                    m_qmu;
  std::condition_variable       m_qcv;
  std::vector<Request*>         m_queue;
  bool                          m_busy = false;
  void*                         m_stage = nullptr;  // pinned rays + results of the batch in flight
  size_t                        m_stageBytes = 0;
  std::mutex                    m_logmu;
  std::string                   m_reported;
};

static_assert(sizeof(CRT_Hit) == sizeof(hrt_hit), "CRT_Hit and hrt_hit must have the same layout");

}  // namespace

ISceneObject* MakeGpuLBVHRT(const char* a_implName, const char* a_buildName, const char* a_layoutName)
{
  return new GpuLBVHRT(a_implName, a_buildName, a_layoutName);
}

// The engine objects behind a scene made by MakeGpuLBVHRT, for the C-ABI calls
// that go beyond ISceneObject (e.g. the renderer frames, hrt_frame_render_rtao).
hrt_scene* GpuLBVHRT_Scene(ISceneObject* scene) { return static_cast<GpuLBVHRT*>(scene)->Scene(); }
hrt_context* GpuLBVHRT_Context(ISceneObject* scene) { return static_cast<GpuLBVHRT*>(scene)->Context(); }

// Batched form for callers that can pass ray arrays; `scene` must come from MakeGpuLBVHRT.
void GpuLBVHRT_NearestHitBatch(ISceneObject* scene, const LiteMath::float4* posAndNear,
                               const LiteMath::float4* dirAndFar, size_t n, CRT_Hit* out)
{
  static_cast<GpuLBVHRT*>(scene)->RayQuery_NearestHitBatch(posAndNear, dirAndFar, n, out);
}
