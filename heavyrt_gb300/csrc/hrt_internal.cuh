// Host-side state of the C ABI shared by its translation units (hrt_api.cu,
// server.cu): contexts, scenes and their geometries, and the helpers that
// build a geometry and report failures.
#pragma once

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "hrt_kernels.cuh"
#include "../../include/hrt.h"

struct hrt_context
{
  int          device = 0;
  int          numSMs = 0;
  cudaStream_t stream = nullptr;
  std::string  lastError;
  std::mutex   mu;
};

namespace hrt
{
namespace api
{

constexpr uint32_t kCounterSlots = 256;

struct Geom
{
  uint32_t     nTris = 0, nVerts = 0, nLeaves = 0;
  float4*      verts = nullptr;
  uint32_t*    keys = nullptr;          // sorted Morton codes
  uint32_t*    vals = nullptr;          // sorted triangle ids (= prim indices)
  uint32_t*    keysUnsorted = nullptr;
  uint32_t*    compressed = nullptr;
  uint32_t*    runStarts = nullptr;
  BVHNode32*   lr = nullptr;
  uint32_t*    lrCount = nullptr;
  PairRec*     recs = nullptr;
  TriRec*      tris = nullptr;
  uint32_t*    sortedIdx = nullptr;
  BuildParams* params = nullptr;
  BuildParams  host{};
  float        buildMs = 0.0f;
  uint64_t     bytes = 0;
  float        box[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  void*        nodes4 = nullptr;  // 4-wide nodes of the scene's layout
  uint32_t     nNodes4 = 0;
  bool         shared = false;    // arrays point into a batch allocation (hrt_add_geoms_triangles3f_batched)
  int          bvh4Merge = 0;     // leaf merge bound the 4-wide nodes were built with
  int          bvh4Collapse = 0;  // HRT_BVH4_COLLAPSE_* the 4-wide nodes were built with (a refit keeps it)
  int          triTest = 0;       // triangle records for HRT_TRI_* (1: vertices, for the watertight test)
  int          mortonFrame = 0;   // HRT_MORTON_* the tree was built in (a refit keeps it)
};

struct Instance
{
  uint32_t geomId = 0;
  float    m[16];     // column-major
  float    inv[12];   // rows 0..2 of the inverse, row-major
  bool     identity = true;
};

}  // namespace api
}  // namespace hrt

struct hrt_scene
{
  using Geom = hrt::api::Geom;
  using Instance = hrt::api::Instance;
  using InstanceDesc = hrt::InstanceDesc;
  using TraceConfig = hrt::TraceConfig;
  hrt_context*          ctx = nullptr;
  std::vector<Geom>     geoms;
  std::vector<Instance> insts;
  std::vector<void*>    batchAllocs;  // device allocations shared by batch-built geometries
  bool                  committed = false;
  int                   layout = HRT_LAYOUT_BVH2;
  int                   bvh4Merge = 0;  // HRT_OPTION_BVH4_MERGE
  int                   bvh4Collapse = 0;  // HRT_OPTION_BVH4_COLLAPSE
  int                   useTlas = 1;    // HRT_OPTION_TLAS
  int                   triTest = 0;    // HRT_OPTION_TRIANGLE_TEST
  int                   mortonFrame = 0;  // HRT_OPTION_MORTON_FRAME
  int                   l2PersistMB = 0;  // HRT_OPTION_L2_PERSIST
  size_t                singleNodeBytes = 0;  // node array of the single instance's geometry
  Geom                  tlas;           // instance tree of the committed scene (nTris = 0: none)
  InstanceDesc*         dInst = nullptr;
  uint32_t              nInstDev = 0;
  // the committed scene is one valid instance under the identity transform
  // (no instance tree): its descriptor, for the single-instance kernel
  bool                  single = false;
  InstanceDesc          singleDesc{};
  uint32_t*             dError = nullptr;
  unsigned long long*   dCounters = nullptr;
  // work counters of the persistent traversal pool: one slot per launch, taken
  // round-robin, so up to kCounterSlots queries on one scene may be in flight
  unsigned int*         dRayCounters = nullptr;
  std::atomic<uint32_t> counterSlot{0};
  TraceConfig           cfg[2];  // [0] nearest, [1] any
  // staging for the host-pointer queries, and the streams that pipeline them
  void*                 stageRays = nullptr;
  void*                 stageOut = nullptr;
  uint64_t              stageCap = 0;
  cudaStream_t          pipe[3] = {nullptr, nullptr, nullptr};
  std::mutex            mu;
};

namespace hrt
{
namespace api
{

// Records msg as the context's last error and returns status.
int fail(hrt_context* ctx, int status, const std::string& msg);
// Maps a CUDA error to HRT_ERR_OUT_OF_MEMORY / HRT_ERR_CUDA with a message.
int cuda_fail(hrt_context* ctx, cudaError_t e, const char* what);
// Frees a geometry's device arrays (not those of a batch-built geometry).
void free_geom(Geom& g);
// Builds one geometry (LBVH, and the 4-wide collapse for a 4-wide layout) on
// s->ctx->stream from host or device arrays; synchronous.  The scene supplies the
// context and the BVH4 merge option; it is not modified.
int build_geometry(hrt_scene* s, Geom& g, const float* vpos, uint64_t nVert, const uint32_t* idx, uint64_t nIdx,
                   uint64_t stride, int layout, int triTest = HRT_TRI_MOLLER_TRUMBORE);
// Traversal view of a geometry under an instance transform (inv12: rows 0..2
// of the inverse; identity when null).
void make_instance_desc(const Geom& g, uint32_t geomId, uint32_t instId, const float* inv12, InstanceDesc& d);
// Column-major 4x4 -> rows 0..2 of its inverse (the reference checker's evaluation).
void inverse4x4(const float* mc, float* inv12);
bool is_identity(const float* m);
// The address at which a kernel reaches host memory in place: the mapped
// device address of page-locked memory; with `pageable`, pageable memory
// itself where the device translates through the host's page tables
// (pageable_access); null otherwise.
void* mapped_host(const void* p, bool pageable = false);
bool pageable_access();
// True when p is a multiple of `bytes` (a power of two).  Kernels read rays
// and write hits as 16-byte vectors, so arrays they access in place must be
// 16-byte aligned; the entry points check this before any launch.
inline bool aligned_to(const void* p, uintptr_t bytes) { return (reinterpret_cast<uintptr_t>(p) & (bytes - 1)) == 0; }

}  // namespace api
}  // namespace hrt

// Returns the mapped status from the enclosing function when a CUDA call fails.
#define HRT_CUDA(ctx, call)                                            \
  do                                                                   \
  {                                                                    \
    cudaError_t e_ = (call);                                           \
    if (e_ != cudaSuccess) return hrt::api::cuda_fail(ctx, e_, #call); \
  } while (0)
