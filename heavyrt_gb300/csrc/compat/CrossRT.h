// Declarations of HeavyRT's ray-query plugin interface (core/CrossRT.h:9-196),
// restated so that the ISceneObject adapter (../scene_rt_adapter.cpp) can be
// built and tested where HeavyRT's sources are absent.  Names, member order,
// signatures and default arguments are the interface's own - an adapter only
// plugs in if they are identical; a real integration puts HeavyRT's core/ first
// on the include path and never sees this file.
#pragma once

#include <cstddef>
#include <cstdint>
#include <unordered_set>

#include "LiteMath.h"

enum BuildQuality
{
  BUILD_LOW    = 0,
  BUILD_MEDIUM = 1,
  BUILD_HIGH   = 2,
  BUILD_REFIT  = 3,
};

// one ray's result: t, primitive / instance / geometry ids, (u, v) in coords[0..1]
struct CRT_Hit
{
  float    t;
  uint32_t primId;
  uint32_t instId;
  uint32_t geomId;
  float    coords[4];
};

constexpr int TREELET_ARR_SIZE = 5;

struct MetricStats
{
  float    avgNC;
  float    avgLC;
  float    avgTC;
  float    avgLJC[TREELET_ARR_SIZE];
  float    avgCMC[TREELET_ARR_SIZE];
  uint32_t avgWSS[TREELET_ARR_SIZE];
  float    avgBLB;
  float    avgSOC;
  float    avgSBL;
  size_t   bvhTotalSize;
  size_t   geomTotalSize;
};

struct ISceneObject
{
  ISceneObject() {}
  virtual ~ISceneObject() {}

  virtual const char* Name() const = 0;
  virtual const char* BuildName() const { return nullptr; }
  virtual void        ClearGeom() = 0;
  virtual uint32_t    AddGeom_Triangles3f(const float* a_vpos3f, size_t a_vertNumber, const uint32_t* a_triIndices,
                                          size_t a_indNumber, BuildQuality a_qualityLevel = BUILD_HIGH,
                                          size_t vByteStride = sizeof(float) * 3) = 0;
  virtual void        UpdateGeom_Triangles3f(uint32_t a_geomId, const float* a_vpos3f, size_t a_vertNumber,
                                             const uint32_t* a_triIndices, size_t a_indNumber,
                                             BuildQuality a_qualityLevel = BUILD_HIGH,
                                             size_t vByteStride = sizeof(float) * 3) = 0;
  virtual void        ClearScene() = 0;
  virtual void        CommitScene(BuildQuality a_qualityLevel = BUILD_MEDIUM) = 0;
  virtual uint32_t    AddInstance(uint32_t a_geomId, const LiteMath::float4x4& a_matrix) = 0;
  virtual void        UpdateInstance(uint32_t a_instanceId, const LiteMath::float4x4& a_matrix) = 0;
  virtual CRT_Hit     RayQuery_NearestHit(LiteMath::float4 posAndNear, LiteMath::float4 dirAndFar) = 0;
  virtual bool        RayQuery_AnyHit(LiteMath::float4 posAndNear, LiteMath::float4 dirAndFar) = 0;

  virtual MetricStats GetStats();
  virtual void        ResetStats();

  virtual uint32_t               GetGeomNum() const { return 0; }
  virtual uint32_t               GetInstNum() const { return 0; }
  virtual const LiteMath::float4* GetGeomBoxes() const { return nullptr; }

protected:
  struct MetricsI
  {
    uint64_t                     NC;
    uint64_t                     LC;
    uint64_t                     LC2;
    uint64_t                     TC;
    uint64_t                     LJC[TREELET_ARR_SIZE];
    uint32_t                     CMC[TREELET_ARR_SIZE];
    std::unordered_set<uint64_t> WSS[TREELET_ARR_SIZE];
    uint64_t                     BLB;
    uint64_t                     SOC;
    uint64_t                     SBL;
    uint32_t                     raysNumber;
    size_t                       bvhTotalSize;
    size_t                       geomTotalSize;
    void                         clear()
    {
      MetricsI zero = {};
      *this = zero;
    }
  } m_stats;
};

ISceneObject* CreateSceneRT(const char* a_implName, const char* a_buildName, const char* a_layoutName);
void          DeleteSceneRT(ISceneObject* a_impl);
