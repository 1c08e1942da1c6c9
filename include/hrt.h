/*
 * hrt.h -- C ABI of the GB300 ray-query engine (LBVH build + BVH2 nearest/any-hit
 * traversal on one GPU).
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (HRT_OK = 0).  The text of the last failure of a context is available from
 * hrt_context_last_error().  The functions mirror HeavyRT's ISceneObject plugin
 * interface (core/CrossRT.h:64-196); the C++ adapter in
 * heavyrt_gb300/csrc/scene_rt_adapter.cpp implements ISceneObject on top of them.
 *
 * Semantics shared by all calls:
 *   - Ray records are two float4 per ray, {posAndNear, dirAndFar}, exactly the
 *     arguments of ISceneObject::RayQuery_NearestHit (core/CrossRT.h:143).
 *   - Hit records are HeavyRT's CRT_Hit (core/CrossRT.h:20-27), 32 bytes:
 *     t, primId, instId, geomId, coords[4] with (u, v) in coords[0..1].  A miss
 *     has t = tFar and primId = instId = geomId = 0xFFFFFFFF.
 *   - primId is the triangle's position in the BVH's Morton-sorted order, as the
 *     reference returns it (core/BVH2CommonRT.cpp:40, REMAP_PRIM_ID off at
 *     core/CrossRT.h:29); hrt_geom_export(HRT_EXPORT_PRIM_INDICES) maps it to the
 *     original triangle index.
 *   - Build calls (add/commit) must not run concurrently with queries on the
 *     same scene; queries may run concurrently with each other.
 *   - Device pointers and `stream` (a cudaStream_t, NULL = legacy default
 *     stream) belong to the caller; the engine owns every BVH buffer.
 */
#ifndef HRT_H
#define HRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- statuses */
#define HRT_OK                  0
#define HRT_ERR_INVALID_ARGUMENT 1  /* null pointer, bad id, size out of range      */
#define HRT_ERR_CUDA            2  /* a CUDA runtime call failed                    */
#define HRT_ERR_OUT_OF_MEMORY   3  /* device allocation refused                     */
#define HRT_ERR_CAPACITY        4  /* input exceeds a format limit (see below)      */
#define HRT_ERR_STATE           5  /* call out of order, e.g. query before commit   */
#define HRT_ERR_TIMEOUT         6  /* a bounded device-side wait gave up            */
#define HRT_ERR_DEVICE_CHECK    7  /* a device-side bounds/consistency check failed */
#define HRT_ERR_UNSUPPORTED     8  /* feature not provided                          */

/* Format limits, checked at build time (HRT_ERR_CAPACITY beyond them):
 *   triangles per geometry  <= 2^24 - 1  (leaf start field, core/raytrace_common.h:38-51)
 *   triangles per leaf      <= 127       (leaf count field; the reference silently
 *                                         corrupts the leaf beyond it, core/builders/lbvh.cpp:382) */
#define HRT_MAX_TRIS_PER_GEOM   ((1u << 24) - 1u)
#define HRT_MAX_TRIS_PER_LEAF   127u

/* Build quality, HeavyRT's BuildQuality (core/CrossRT.h:9-15).  All values
 * build the same LBVH; BUILD_REFIT is accepted by hrt_update_geom_triangles3f. */
#define HRT_BUILD_LOW    0
#define HRT_BUILD_MEDIUM 1
#define HRT_BUILD_HIGH   2
#define HRT_BUILD_REFIT  3

typedef struct hrt_context hrt_context;
typedef struct hrt_scene   hrt_scene;

/* CRT_Hit, core/CrossRT.h:20-27. */
typedef struct hrt_hit
{
  float    t;
  uint32_t primId;
  uint32_t instId;
  uint32_t geomId;
  float    coords[4];
} hrt_hit;

/* ---------------------------------------------------------------- context */

/* Opens the engine on CUDA device `device`.  No reference counterpart: the
 * reference runs on the host only. */
int hrt_context_create(int device, hrt_context** out);
int hrt_context_destroy(hrt_context* ctx);
/* Text of the most recent failure on this context ("" if none). */
const char* hrt_context_last_error(const hrt_context* ctx);
/* Static text for a status code. */
const char* hrt_status_string(int status);
/* Engine version string. */
const char* hrt_version(void);

/* ---------------------------------------------------------------- scenes */

/* Replaces CreateSceneRT(a_implName, a_buildName, a_layoutName) for the
 * "BVH2Common" + "cbvh_lbvh" combination (core/FactoryRT.cpp:29-78,
 * core/CrossRT.h:195).  buildName may be NULL or any of HeavyRT's builder
 * strings that select the LBVH ("cbvh_lbvh", "lbvh", "cbvh_lbvh_gpu");
 * anything else is HRT_ERR_UNSUPPORTED. */
int hrt_scene_create(hrt_context* ctx, const char* buildName, hrt_scene** out);
/* Replaces DeleteSceneRT (core/CrossRT.h:196). */
int hrt_scene_destroy(hrt_scene* scene);

/* Node layout of a scene's acceleration structures, HeavyRT's a_layoutName
 * argument of CreateSceneRT (core/CrossRT.h:195).  Chosen before the first
 * geometry is added (HRT_ERR_STATE afterwards).
 *   BVH2      binary LBVH, 64-byte child-pair records (default; the
 *             reference's BVH2CommonRT decisions, bit-exact)
 *   BVH4_F32  4-wide collapse (core/builders/cbvh.cpp:226-311), FP32 boxes, 128 B nodes
 *   BVH4_F16  4-wide, FP16 boxes rounded outward, 64 B nodes
 *   BVH4_Q8   4-wide, 8-bit offsets against a per-node FP32 frame with
 *             power-of-two scales, rounded outward, 64 B nodes
 * Quantised boxes contain their FP32 boxes, so they can only add node visits;
 * the triangle test is the same in every layout. */
#define HRT_LAYOUT_BVH2     0
#define HRT_LAYOUT_BVH4_F32 1
#define HRT_LAYOUT_BVH4_F16 2
#define HRT_LAYOUT_BVH4_Q8  3
int hrt_scene_set_layout(hrt_scene* scene, int layout);
int hrt_scene_get_layout(const hrt_scene* scene, int* layout);

/* Build options (applied to geometry added afterwards).  No reference
 * counterpart beyond the collapse rule itself.
 *   HRT_OPTION_BVH4_MERGE  0: a node whose two children are leaves becomes
 *                          one leaf (BVH2ToBVH4, core/builders/cbvh.cpp:242-255);
 *                          M in 1..64: a subtree of at most M triangles becomes
 *                          one leaf (1 never merges). */
#define HRT_OPTION_BVH4_MERGE 1
/*   HRT_OPTION_TLAS        1 (default): hrt_commit_scene builds an instance tree
 *                          (a binary LBVH over the instances' world-space boxes,
 *                          the role of the reference's TLAS, core/BVH2CommonRT_host.cpp:118-129)
 *                          when the scene has two or more instances, and queries
 *                          traverse it and the instances' trees in one kernel;
 *                          0: every instance is traversed in instance order.
 *                          Results are the same either way, except which of two
 *                          instances wins an exact tie in t. */
#define HRT_OPTION_TLAS 2
/*   HRT_OPTION_TRIANGLE_TEST  the ray-triangle test of every geometry of the
 *                          scene, chosen before the first geometry is added
 *                          (HRT_ERR_STATE afterwards):
 *     HRT_TRI_MOLLER_TRUMBORE (default) HeavyRT's test (core/BVH2CommonRT.cpp:9-47):
 *                          Moller-Trumbore with 1e-6 barycentric slack,
 *                          results bit-exact with the reference;
 *     HRT_TRI_WATERTIGHT   the watertight test of Woop, Benthin & Wald (JCGT
 *                          2013) in FP32 with exact edge-function signs: no
 *                          ray passes between two triangles that share an
 *                          edge, and no hit is accepted outside a triangle.
 *                          Hits agree with the reference except for rays
 *                          within about 1e-6 (in barycentric terms) of an
 *                          edge.  The scene's triangle records then hold the
 *                          three vertices instead of a vertex and two edges. */
#define HRT_OPTION_TRIANGLE_TEST 3
#define HRT_TRI_MOLLER_TRUMBORE  0
#define HRT_TRI_WATERTIGHT       1
/*   HRT_OPTION_L2_PERSIST  value > 0: the node array of a scene of one
 *                          untransformed geometry is kept in L2 for its
 *                          queries: the process's persisting-L2 set-aside on
 *                          the scene's device becomes `value` MiB (capped by
 *                          the device's maximum; a context-wide limit that
 *                          ends with the process), and each traversal launch
 *                          marks the node array persisting through an
 *                          access-policy window (the share that fits the
 *                          set-aside).  0 (default): no window.  Results
 *                          never depend on it. */
#define HRT_OPTION_L2_PERSIST 4
/*   HRT_OPTION_MORTON_FRAME  the grid the Morton codes of geometry added
 *                          afterwards are quantised on:
 *     HRT_MORTON_PER_AXIS  (default) HeavyRT's ZIndexMultCoeff
 *                          (core/builders/lbvh.cpp:41-51): each axis of the
 *                          scene box divided into 1024 cells; the build is
 *                          the reference's bit for bit;
 *     HRT_MORTON_CUBIC     one scale for all three axes, that of the longest
 *                          extent (cubic cells), so a flat or elongated scene
 *                          does not split its short axes as often as its long
 *                          ones.  The same LBVH otherwise; a different tree, so
 *                          hits equal the reference's except at ties within
 *                          1e-5 relative t. */
#define HRT_OPTION_MORTON_FRAME 5
#define HRT_MORTON_PER_AXIS     0
#define HRT_MORTON_CUBIC        1
/*   HRT_OPTION_BVH4_COLLAPSE  which binary nodes a 4-wide node of geometry
 *                          added afterwards takes as its (up to) four slots:
 *     HRT_BVH4_COLLAPSE_EVEN_DEPTH  (default) BVH2ToBVH4's rule
 *                          (core/builders/cbvh.cpp:226-311): the grandchildren,
 *                          so the 4-wide nodes are the binary nodes at even
 *                          depth;
 *     HRT_BVH4_COLLAPSE_LARGEST_FIRST  start from the two children and twice
 *                          open the internal slot with the most leaves under
 *                          it (the leftmost of equals) into its two children,
 *                          so big subtrees descend faster and small ones are
 *                          not split early.  It depends on the tree's shape
 *                          alone, so a refit keeps it.  The merge option
 *                          applies to the internal slots left after the
 *                          openings.  Another 4-wide tree over the same
 *                          binary tree: hits equal the reference's except at
 *                          ties within 1e-5 relative t. */
#define HRT_OPTION_BVH4_COLLAPSE          6
#define HRT_BVH4_COLLAPSE_EVEN_DEPTH      0
#define HRT_BVH4_COLLAPSE_LARGEST_FIRST   1
int hrt_scene_set_option(hrt_scene* scene, int option, int value);

/* ISceneObject::ClearGeom (core/CrossRT.h:82): drops every geometry and instance. */
int hrt_clear_geom(hrt_scene* scene);

/* ISceneObject::AddGeom_Triangles3f (core/CrossRT.h:94; reference implementation
 * core/BVH2CommonRT_host.cpp:66-98).  Host arrays: vpos has nVert vertices of
 * vByteStride bytes (0 means 12), xyz first; idx has nIdx indices (3 per
 * triangle).  The data is copied; the LBVH is built on the GPU before the call
 * returns.  *geomId receives the new geometry id. */
int hrt_add_geom_triangles3f(hrt_scene* scene, const float* vpos, uint64_t nVert, const uint32_t* idx, uint64_t nIdx,
                             int quality, uint64_t vByteStride, uint32_t* geomId);

/* ISceneObject::UpdateGeom_Triangles3f (core/CrossRT.h:105; every reference
 * implementation stubs it, e.g. core/BVH2CommonRT_host.cpp:100-103).
 *   quality == HRT_BUILD_REFIT: the vertices moved, the triangles did not
 *     (same vertex and index counts, same index buffer): the tree's topology
 *     and sorted order are kept and every box and record is recomputed on the
 *     GPU (the reference's BUILD_REFIT intent, core/CrossRT.h:13); works for
 *     batch-built geometries too.
 *   any other quality: the geometry is rebuilt from the new arrays (any size)
 *     under the same id.
 * Either way the scene must be committed again before the next query (the
 * instance tree and descriptors follow the new geometry). */
int hrt_update_geom_triangles3f(hrt_scene* scene, uint32_t geomId, const float* vpos, uint64_t nVert,
                                const uint32_t* idx, uint64_t nIdx, int quality, uint64_t vByteStride);

/* ISceneObject::ClearScene (core/CrossRT.h:110): drops instances, keeps geometry. */
int hrt_clear_scene(hrt_scene* scene);

/* ISceneObject::AddInstance (core/CrossRT.h:123; core/BVH2CommonRT_host.cpp:131-164).
 * m: 16 floats, column-major 4x4 (LiteMath::float4x4 layout). */
int hrt_add_instance(hrt_scene* scene, uint32_t geomId, const float m[16], uint32_t* instId);

/* ISceneObject::UpdateInstance (core/CrossRT.h:130). */
int hrt_update_instance(hrt_scene* scene, uint32_t instId, const float m[16]);

/* ISceneObject::CommitScene (core/CrossRT.h:115; core/BVH2CommonRT_host.cpp:118-129):
 * finishes instancing.  Queries are valid after it returns. */
int hrt_commit_scene(hrt_scene* scene, int quality);

/* ---------------------------------------------------------------- queries */

/* Batched ISceneObject::RayQuery_NearestHit (core/CrossRT.h:143; reference
 * traversal core/BVH2CommonRT.cpp:49-141,228-279).  Device arrays: rays has
 * n records of 8 floats, hits has n records.  Asynchronous on `stream`. */
int hrt_query_nearest(hrt_scene* scene, const float* rays, uint64_t n, hrt_hit* hits, void* stream);

/* Batched ISceneObject::RayQuery_AnyHit (core/CrossRT.h:151).  The reference's
 * BVH2CommonRT stubs it (core/BVH2CommonRT.cpp:281-292); the semantics follow its
 * siblings (core/BVH2CommonRTStacklessLBVH.cpp:161-165,235-240): 1 if some
 * triangle passes the ray-triangle test with tNear < t < tFar.  out: n bytes. */
int hrt_query_any(hrt_scene* scene, const float* rays, uint64_t n, uint8_t* out, void* stream);

/* Same as the two calls above with HOST arrays; the results are in place when
 * the call returns.  Page-locked arrays (hrt_host_alloc, cudaHostAlloc,
 * cudaHostRegister) at a 16-byte boundary are used where they are: the
 * traversal reads their rays over the host link and writes its results
 * straight into them.  On devices that translate through the host's page
 * tables (Grace-based systems) pageable rays are read in place too.  Other
 * host memory is copied in and out; such batches
 * above 2^18 rays run as chunks whose copies overlap the traversal of other
 * chunks.  The device-pointer calls above want rays (and hits) at a 16-byte
 * boundary and return HRT_ERR_INVALID_ARGUMENT otherwise. */
int hrt_query_nearest_host(hrt_scene* scene, const float* rays, uint64_t n, hrt_hit* hits);
int hrt_query_any_host(hrt_scene* scene, const float* rays, uint64_t n, uint8_t* out);

/* The host-pointer queries, enqueued on `stream` instead of waited for: the
 * results are in place once the stream has reached them.  Page-locked arrays
 * are used in place as above, and so are pageable rays on devices that
 * translate through the host's page tables (Grace-based systems): there the
 * traversal reads the caller's ray array while the stream runs, so its
 * contents must not change until the stream is done.  Other memory goes
 * through stream-ordered device allocations (a pageable result array makes
 * the final copy synchronous).  Queries on different streams overlap, e.g.
 * one batch's result copy with the next batch's traversal.  The arrays must
 * stay valid until the stream is done. */
int hrt_query_nearest_host_async(hrt_scene* scene, const float* rays, uint64_t n, hrt_hit* hits, void* stream);
int hrt_query_any_host_async(hrt_scene* scene, const float* rays, uint64_t n, uint8_t* out, void* stream);

/* Reads and clears the scene's device-side check word after asynchronous
 * queries (call once their streams are synchronised): HRT_ERR_DEVICE_CHECK if
 * a ray ran out of its step budget or the stack bound, HRT_OK otherwise. */
int hrt_scene_check(hrt_scene* scene);

/* Launch shape of the traversal kernel, per query kind (0 nearest, 1 any);
 * results never depend on it.  No reference counterpart (the reference runs
 * one ray per virtual call with an 80-entry stack, core/raytrace_common.h:34).
 * Defaults: 128 threads, persistent pool, 16 steps between refills, refill at
 * 24 idle lanes, the whole stack in shared memory.
 * imageWidth is a property of the rays the kind's queries pass (the
 * autotuner keeps it).
 * stackEntries: traversal stack entries per ray kept in shared memory; deeper
 * entries spill to the thread's local memory, so any value is correct for any
 * tree.  0, or a value at or above the layout's depth bound (32 binary, 48
 * 4-wide, +32 with an instance tree), keeps the whole stack in shared memory. */
#define HRT_MAX_STACK_ENTRIES 128
typedef struct hrt_trace_config
{
  int threadsPerBlock; /* 64, 128 or 256                                          */
  int persistent;      /* 1: persistent warp pool that refills idle lanes; 0: one thread per ray */
  int stepsPerRefill;  /* traversal steps between refill checks (1..1024)        */
  int refillLanes;     /* a warp refills when at least this many lanes are idle (1..32) */
  int stackEntries;    /* short-stack entries in shared memory (0..HRT_MAX_STACK_ENTRIES) */
  int imageWidth;      /* > 0: the rays form row-major images this many rays wide (as a
                          renderer's eye rays do), and the traversal takes them in tiles of
                          4 x 8 pixels so that neighbouring pixels trace together; results
                          still go to each ray's index.  0: rays taken in the order given */
} hrt_trace_config;
int hrt_scene_set_trace_config(hrt_scene* scene, int kind, const hrt_trace_config* config);
int hrt_scene_get_trace_config(const hrt_scene* scene, int kind, hrt_trace_config* config);

/* Traversal work of a batch, the quantity behind ISceneObject::GetStats
 * (core/CrossRT.h:154, core/FactoryRT.cpp:82-101): counters[0] = node pairs
 * fetched (HeavyRT counts 2 nodes, 64 bytes, per pair), counters[1] = triangle
 * tests.  kind: 0 nearest, 1 any.  Device rays; synchronous. */
int hrt_query_counters(hrt_scene* scene, int kind, const float* rays, uint64_t n, uint64_t counters[2], void* stream);

/* ---------------------------------------------------------------- batches of scenes
 * Many small scenes served together: their geometries are built by one
 * segmented LBVH build and their rays traced by one kernel launch.  No
 * single reference call corresponds; each geometry and each hit is exactly
 * what one AddGeom_Triangles3f (core/BVH2CommonRT_host.cpp:66-98) and one
 * RayQuery_NearestHit / RayQuery_AnyHit per scene would give. */

/* AddGeom_Triangles3f for `count` geometries at once.  Host arrays:
 * geometry i has vertices vertOffsets[i] .. vertOffsets[i+1]-1 of vpos
 * (vByteStride bytes each, 0 means 12) and indices idxOffsets[i] ..
 * idxOffsets[i+1]-1 of idx (a multiple of 3 each), its indices counting from
 * its own first vertex.  Both offset arrays have count+1 entries starting at
 * 0.  The geometries get ids *firstGeomId .. *firstGeomId+count-1; their
 * device memory is shared and freed by hrt_clear_geom / hrt_scene_destroy.
 * Limits: each geometry HRT_MAX_TRIS_PER_GEOM, the batch
 * HRT_MAX_TRIS_PER_BATCH triangles and 2^32-1 vertices. */
#define HRT_MAX_TRIS_PER_BATCH ((1u << 30) - 1u)
int hrt_add_geoms_triangles3f_batched(hrt_scene* scene, uint32_t count, const float* vpos, const uint64_t* vertOffsets,
                                      const uint32_t* idx, const uint64_t* idxOffsets, int quality,
                                      uint64_t vByteStride, uint32_t* firstGeomId);

/* One traversal launch.  rays/out as for hrt_query_nearest / hrt_query_any.
 * With rayOffsets == NULL every ray is traced against the whole scene; else
 * rays rayOffsets[k] .. rayOffsets[k+1]-1 are traced against instance
 * segInst[k] only (as a scene holding just that instance would trace them;
 * the hit's instId is segInst[k]).  rayOffsets (nSeg+1 entries, ascending, 0
 * first, n last) and segInst (nSeg entries) are device arrays; a ray whose
 * instance id is out of range is a miss. */
typedef struct hrt_query_desc
{
  int             kind;        /* 0 nearest (out: hrt_hit[n]), 1 any (out: uint8_t[n]) */
  const float*    rays;        /* device, 8 floats per ray                             */
  uint64_t        n;
  const uint32_t* rayOffsets;  /* device or NULL                                       */
  const uint32_t* segInst;     /* device                                               */
  uint32_t        nSeg;
  void*           out;         /* device                                               */
} hrt_query_desc;
int hrt_query_multi(hrt_scene* scene, const hrt_query_desc* query, void* stream);

/* Captured query sequences: the launches of `count` queries (in order) are
 * recorded once into a CUDA graph and replayed by hrt_graph_launch with one
 * call.  The descriptors' device buffers must stay valid while the graph
 * exists; their contents may change between launches.  A graph keeps its own
 * work counters, so different graphs may run concurrently; one graph runs
 * one launch at a time.  The scene must not be rebuilt or recommitted while
 * one of its graphs exists. */
typedef struct hrt_graph hrt_graph;
int hrt_graph_create(hrt_scene* scene, const hrt_query_desc* queries, uint32_t count, hrt_graph** graph);
int hrt_graph_launch(hrt_graph* graph, void* stream);
int hrt_graph_destroy(hrt_graph* graph);

/* Launch-shape autotuner: times `query` (repeats timed runs after one
 * warm-up) under every trace configuration of a fixed grid (64/128/256
 * threads; one ray per thread, or the persistent pool with 4..64 steps per
 * refill and 2..32 idle lanes to refill), then the best of those with 16, 24,
 * 32, 48 and 64 shared-memory stack entries; sets the fastest as the scene's
 * configuration for query->kind, and returns it with its mean time in ms.
 * Synchronous; overwrites query->out (with identical results). */
int hrt_scene_autotune(hrt_scene* scene, const hrt_query_desc* query, int repeats, hrt_trace_config* best,
                       float* bestMs);

/* ---------------------------------------------------------------- serving
 * A request loop over scenes kept resident in device memory.  No reference
 * counterpart (HeavyRT's renderers call ISceneObject per ray on one scene).
 *
 * Scenes are built on arrival by the server's builder thread and admitted
 * against a device-memory budget: when a new scene does not fit, idle
 * evictable scenes are evicted, least recently used first.  Ray requests
 * (host arrays) are queued; whenever one of the server's batch slots is free,
 * a dispatcher packs every queued request whose scene is ready (in arrival
 * order, up to the slot's capacity) into one batch and traces it with one
 * segmented launch per query kind on the slot's own stream.  Requests that
 * arrive while batches are on the GPU join the next free slot, and the
 * copies and traversals of successive batches overlap.  A request's results
 * do not depend on the requests it was batched with.
 *
 * Host ray / result buffers must stay valid until the request is waited for;
 * page-locked buffers (hrt_host_alloc) copy at full link speed.  Every ticket
 * must be waited for exactly once.  Scene ids of evicted or removed scenes
 * are never valid again. */
typedef struct hrt_server hrt_server;

typedef struct hrt_server_config
{
  uint64_t memoryBudget;     /* device bytes for scenes + batch slots; 0 = 150e9          */
  uint64_t slotRays;         /* rays per batch slot = largest request; 0 = 8,388,608       */
  uint32_t slots;            /* batches in flight, 1..16; 0 = 3                            */
  uint32_t maxScenes;        /* resident scene capacity, <= 65536; 0 = 4096                */
  uint32_t maxBatchRequests; /* requests per batch; 0 = 1024                               */
  int      layout;           /* HRT_LAYOUT_* of every scene                                */
  int      bvh4Merge;        /* HRT_OPTION_BVH4_MERGE value for 4-wide layouts             */
  int      mortonFrame;      /* HRT_MORTON_* grid of every scene's build                   */
  int      bvh4Collapse;     /* HRT_BVH4_COLLAPSE_* rule of every scene's 4-wide nodes     */
} hrt_server_config;

/* Result of one request; times in seconds since the server was created. */
typedef struct hrt_request_info
{
  int      status;         /* HRT_OK, or why the request failed                    */
  uint32_t batch;          /* sequence number of the batch that traced it          */
  uint32_t batchRequests;  /* requests in that batch                               */
  uint64_t batchRays;      /* rays in that batch                                   */
  double   tSubmit, tStart, tDone;
} hrt_request_info;

typedef struct hrt_server_stats
{
  uint64_t requests, rays, batches, builds, evictions, failed;
  uint64_t residentBytes, peakResidentBytes;  /* held against the budget        */
  uint32_t scenesResident, queued;
} hrt_server_stats;

#define HRT_SCENE_BUILDING 0
#define HRT_SCENE_READY    1
#define HRT_SCENE_FAILED   2
#define HRT_SCENE_EVICTED  3  /* evicted, removed or never existed */

int hrt_server_create(hrt_context* ctx, const hrt_server_config* config, hrt_server** server);
/* Finishes queued builds and requests, then frees everything. */
int hrt_server_destroy(hrt_server* server);
/* Queues the build of a scene of one triangle geometry under the identity
 * (arguments as hrt_add_geom_triangles3f; the arrays are copied to the device
 * before the call returns, at full link speed when they are page-locked).
 * Requests may be submitted at once; they run when the build is done.
 * evictable = 0 keeps the scene until it is removed.
 * HRT_ERR_OUT_OF_MEMORY when it cannot fit the budget even after evictions. */
int hrt_server_add_scene(hrt_server* server, const float* vpos, uint64_t nVert, const uint32_t* idx, uint64_t nIdx,
                         uint64_t vByteStride, int evictable, uint32_t* sceneId);
/* HRT_SCENE_* state; waits up to timeoutSeconds (< 0: no limit) while building. */
int hrt_server_scene_state(hrt_server* server, uint32_t sceneId, double timeoutSeconds, int* state);
/* Frees a ready scene with no requests queued or in flight (HRT_ERR_STATE otherwise). */
int hrt_server_remove_scene(hrt_server* server, uint32_t sceneId);
/* Queues a request: n rays (host, 8 floats each) against one scene; kind 0
 * writes hrt_hit[n] to out, kind 1 uint8_t[n].  Both arrays must stay valid
 * until the request is waited for.  A request batched alone whose rays are
 * page-locked is traced from them in place (its any-hit flags written in
 * place when out is page-locked); otherwise the rays are copied in.  Ray
 * batches run at the highest stream priority, scene builds at the lowest. */
int hrt_server_submit(hrt_server* server, uint32_t sceneId, int kind, const float* rays, uint64_t n, void* out,
                      uint64_t* ticket);
/* Waits for a request (timeoutSeconds < 0: no limit; HRT_ERR_TIMEOUT leaves the
 * ticket valid); returns the request's status and fills info. */
int hrt_server_wait(hrt_server* server, uint64_t ticket, double timeoutSeconds, hrt_request_info* info);
int hrt_server_get_stats(hrt_server* server, hrt_server_stats* stats);
/* Bytes a scene of nVert vertices and nTris triangles reserves against the
 * budget while it is built (its arrays, the build's transient arrays and the
 * device copy of its inputs, for vertices of up to 16 bytes); once built it
 * holds its actual, smaller size. */
int hrt_server_scene_bytes(const hrt_server* server, uint64_t nVert, uint64_t nTris, uint64_t* bytes);

/* ---------------------------------------------------------------- ray generation on the GPU
 * A frame's rays made where they are traced, so that neither the eye rays
 * nor the AO rays chained from their hits cross the host link.  Output arrays
 * are device memory (8 floats per ray); asynchronous on `stream` unless noted. */

/* The renderers' eye rays: RTAO::kernel_InitEyeRay (examples/02_rtao/rtao.cpp:133-144,
 * examples/01_eye_rays/eye_ray.cpp:26-47) with EyeRayDirNormalized / transform_ray3f
 * (examples/render_common.h:6-36).  projInv, worldViewInv: column-major 4x4;
 * one ray per pixel centre, row-major (pixel x, y at index y * width + x). */
int hrt_gen_eye_rays(hrt_context* ctx, const float projInv[16], const float worldViewInv[16], uint32_t width,
                     uint32_t height, float tNear, float tFar, float* rays, void* stream);

/* Pinhole camera at eye looking at target (up hint, vertical field of view
 * fovDeg): the benchmark workloads' eye rays, equal to the host generator's
 * (heavyrt_gb300/workload.py camera_rays) bit for bit. */
int hrt_gen_pinhole_rays(hrt_context* ctx, const float eye[3], const float target[3], const float up[3], float fovDeg,
                         uint32_t width, uint32_t height, float tmin, float tmax, float* rays, void* stream);

/* Ambient-occlusion rays from primary hits (device eye rays and their hits):
 * for every hit, perHit cosine-weighted directions about the hit triangle's
 * geometric normal turned toward the eye, from the PCG32 stream (seed, hit's
 * eye-ray index + 16); origin = hit point + offset * normal, tmin 0, tmax =
 * length.  Hits are compacted in eye-ray order, as the host generator
 * (heavyrt_gb300/workload.py ao_rays) orders them; owner (device, optional)
 * receives each AO ray's eye-ray index.  Needs identity instances.
 * Synchronous: *count receives the number of AO rays (HRT_ERR_CAPACITY when
 * it exceeds capacity). */
int hrt_gen_ao_rays(hrt_scene* scene, uint64_t seed, const float* eyeRays, const hrt_hit* hits, uint64_t nEye,
                    uint32_t perHit, float length, float offset, float* aoRays, uint32_t* owner, uint64_t capacity,
                    uint64_t* count, void* stream);

/* ---------------------------------------------------------------- renderer frames
 * Whole frames of HeavyRT's two example renderers on the device (replacing
 * EyeRayCaster::CastRaySingleBlock, examples/01_eye_rays/eye_ray_host.cpp:332-362,
 * and RTAO::CalcAOBlock, examples/02_rtao/rtao.cpp:28-44, over this engine's
 * scene): rays generated, traced and shaded on the GPU, every value equal bit
 * for bit to the renderers' own kernels run on the same hits.  A frame object
 * owns its buffers (grown on demand) and is used by one thread at a time.
 * Colours: width * height uint32 RGBA, row-major pixels (x, y at
 * y * width + x), in device memory (written by the kernels) or in host memory
 * (copied there at the end of the frame, which then synchronises `stream`).  Rays are traced in EyeRayCaster's packed order
 * (kernel_PackXY, eye_ray.cpp:106-134: 4x4 blocks in 2x2 super-blocks) when
 * both sides are multiples of 8, row by row otherwise; the images are the same. */
typedef struct hrt_frame hrt_frame;
int hrt_frame_create(hrt_context* ctx, hrt_frame** out);
int hrt_frame_destroy(hrt_frame* frame);

/* EyeRayCaster frame (eye_ray.cpp:10-74): kernel_InitEyeRay (tNear 0, tFar
 * MAXFLOAT), nearest hit, colour 0 on a miss, else the renderer's 20-entry
 * palette at primId % 20 (primId = the hit's sorted position, as the
 * reference's BVH2CommonRT returns it).  Asynchronous on `stream`. */
int hrt_frame_render_eye(hrt_frame* frame, hrt_scene* scene, const float projInv[16], const float worldViewInv[16],
                         uint32_t width, uint32_t height, uint32_t* colors, void* stream);

/* RTAO's quasi-random AO samples (RTAO::InitQMCTable, examples/02_rtao/rtao_host.cpp:383-414):
 * hrt_rtao_qmc_table: the 4 x 31 direction numbers of initQuasirandomGenerator
 * (core/common/qmc_sobol_niederreiter.cpp:179-186); hrt_rtao_qmc_tile: the
 * 128 x 128 texel tile, raysPerPixel (r1, r2) pairs per texel (2 floats each,
 * texel (x, y) at (y * 128 + x) * raysPerPixel), host memory, no context. */
#define HRT_AO_TILE_SIZE          128
#define HRT_MAX_AO_RAYS_PER_PIXEL 1024
int hrt_rtao_qmc_table(uint32_t* table);
int hrt_rtao_qmc_tile(uint32_t raysPerPixel, float* tile);

/* The RTAO frame's inputs that outlive a frame: the sample tile (host memory,
 * 128 * 128 * raysPerPixel float pairs, e.g. from hrt_rtao_qmc_tile; sets the
 * frame's raysPerPixel) and each geometry's vertex normals (float4 per vertex
 * in the geometry's vertex order, host or device memory; RTAO::m_vNorm4f). */
int hrt_frame_set_ao_tile(hrt_frame* frame, const float* tile, uint32_t raysPerPixel);
int hrt_frame_set_normals(hrt_frame* frame, uint32_t geomId, const float* normals, uint64_t nVerts);

/* RTAO's camera and AO settings (RTAO::m_projInv, m_worldViewInv, m_zNearFar,
 * m_aoMaxRadius, m_power); matrices column-major. */
typedef struct hrt_rtao_params
{
  float    projInv[16];
  float    worldViewInv[16];
  float    zNear, zFar;
  uint32_t width, height;
  float    aoMaxRadius;
  float    power;
} hrt_rtao_params;

/* RTAO frame (RTAO::CalcAO, rtao.cpp:46-60, for every pixel): kernel_InitEyeRay,
 * nearest hit, kernel_TraceEyeRay2's hit point and packed shading normal
 * (vertex normals of the hit triangle through normMatrices[instId]: 16 floats
 * per instance, column-major, host memory; RTAO::m_normMatrices),
 * kernel_InitAORay's raysPerPixel rays for every pixel with a hit, their
 * occlusion (any hit), kernel_AO2Color.  Synchronises `stream` once (to size
 * the AO launch); the rest is asynchronous. */
int hrt_frame_render_rtao(hrt_frame* frame, hrt_scene* scene, const hrt_rtao_params* params, const float* normMatrices,
                          uint32_t* colors, void* stream);

/* Device buffers of the frame's last render, valid until the next one:
 *   EYE_RAYS   8 floats per traced eye ray, in trace order      (count = pixels)
 *   RAY_PIXEL  uint32 pixel index of each traced eye ray       (count = pixels)
 *   EYE_HITS   hrt_hit per traced eye ray                       (count = pixels)
 *   POSITIONS  float4 per pixel: hit point + packed normal in w (RTAO; y = 1e7 without a hit)
 *   VISIBILITY float per pixel: unoccluded AO samples           (RTAO; 0 without a hit)
 *   AO_PIXEL   uint32 pixel of each AO slot (pixels with a hit, trace order)
 *   AO_RAYS    8 floats per AO ray: slot s, sample z at s * raysPerPixel + z
 *   AO_HITS    uint8 occlusion flag per AO ray */
#define HRT_FRAME_EYE_RAYS   0
#define HRT_FRAME_RAY_PIXEL  1
#define HRT_FRAME_EYE_HITS   2
#define HRT_FRAME_POSITIONS  3
#define HRT_FRAME_VISIBILITY 4
#define HRT_FRAME_AO_PIXEL   5
#define HRT_FRAME_AO_RAYS    6
#define HRT_FRAME_AO_HITS    7
int hrt_frame_get_buffer(const hrt_frame* frame, int which, const void** data, uint64_t* count);
/* The same buffer copied into dst (host or device memory, capacityBytes long)
 * after the device has finished; *bytes receives its size (HRT_ERR_CAPACITY
 * when dst is too small).  Synchronous. */
int hrt_frame_read_buffer(const hrt_frame* frame, int which, void* dst, uint64_t capacityBytes, uint64_t* bytes);

/* ---------------------------------------------------------------- on-disk formats */

/* VSGF meshes, HeavyRT's binary mesh files (examples/loader/cmesh.cpp:80-173):
 * a 24-byte header {u64 file size, u32 vertices, u32 indices, u32 materials,
 * u32 flags}, float4 positions, float4 normals (absent with flag 8), float4
 * tangents (with flag 1), float2 texture coordinates, u32 indices, one u32
 * material per triangle.  Host-only; no context needed.
 * hrt_vsgf_info: counts and flags (HRT_ERR_INVALID_ARGUMENT for a missing,
 * truncated or malformed file).  hrt_vsgf_read: positions (nVert float4) and
 * indices into caller buffers; normals too when norm4 is not NULL (zeros when
 * the file has none).  hrt_vsgf_write: positions + indices (no normals). */
int hrt_vsgf_info(const char* path, uint64_t* nVert, uint64_t* nIdx, uint32_t* flags);
int hrt_vsgf_read(const char* path, float* vpos4, uint32_t* idx, float* norm4);
int hrt_vsgf_write(const char* path, const float* vpos4, uint64_t nVert, const uint32_t* idx, uint64_t nIdx);

/* BVH blobs: every device array of a built geometry in one file, so that a
 * geometry is restored by copies alone, without a build (a warm start for
 * resident scenes).  A blob loads only into a scene of the layout and
 * triangle test it was built for (HRT_ERR_STATE otherwise); hrt_geom_load
 * appends a geometry and returns its id.  The geometry keeps the build
 * options it was built with (merge bound, collapse rule, Morton frame), so a
 * later refit rebuilds it the same way whatever the loading scene's options. */
int hrt_geom_save(const hrt_scene* scene, uint32_t geomId, const char* path);
int hrt_geom_load(hrt_scene* scene, const char* path, uint32_t* geomId);

/* ---------------------------------------------------------------- scene info */

/* ISceneObject::GetGeomNum / GetInstNum / GetGeomBoxes (core/CrossRT.h:163-165). */
int hrt_get_geom_num(const hrt_scene* scene, uint32_t* out);
int hrt_get_inst_num(const hrt_scene* scene, uint32_t* out);
/* boxes: 8 floats per geometry (boxMin float4, boxMax float4), host memory. */
int hrt_get_geom_boxes(const hrt_scene* scene, float* boxes, uint32_t capacity);

/* Per-geometry build information: out[0] triangles, out[1] leaves, out[2]
 * internal node pairs, out[3] device bytes held; build_ms = GPU time of the
 * LBVH build kernels. */
int hrt_geom_info(const hrt_scene* scene, uint32_t geomId, uint64_t out[4], float* build_ms);

/* Copies an intermediate or final array of a geometry's build to host memory,
 * for parity checks against HeavyRT's builder.  capacityBytes = size of dst;
 * *sizeBytes receives the bytes the array holds (dst may be NULL to query). */
#define HRT_EXPORT_SCENE_BOX       0 /* 12 floats: bboxMin4, bboxMax4, zIndexScale4 (lbvh.cpp:41-51,228-263) */
#define HRT_EXPORT_MORTON_SORTED   1 /* uint2[N] (code, triId) after the stable sort (lbvh.cpp:755)        */
#define HRT_EXPORT_COMPRESSED      2 /* uint32[L] unique codes (lbvh.cpp:302-319)                          */
#define HRT_EXPORT_RUN_STARTS      3 /* uint32[L] first sorted position of each code (lbvh.cpp:302-319)    */
#define HRT_EXPORT_LR_NODES        4 /* BVHNode[2L-1] Karras + refit tree, LR format (lbvh.cpp:350-489)    */
#define HRT_EXPORT_LR_COUNTS       5 /* uint32[2L-1] descendant node counts (lbvh.cpp:443-489)             */
#define HRT_EXPORT_PRIM_INDICES    6 /* uint32[N] original triangle of each sorted position                */
#define HRT_EXPORT_SORTED_INDICES  7 /* uint32[3N] index buffer in sorted order (BVH2CommonRT_host.cpp:45-64) */
#define HRT_EXPORT_MORTON_UNSORTED 8 /* uint2[N] (code, triId) before the sort (lbvh.cpp:259-287)           */
#define HRT_EXPORT_NODES4          9 /* the 4-wide nodes of a BVH4 layout, raw (128 or 64 bytes each)      */
#define HRT_EXPORT_PAIR_RECORDS   10 /* the binary layout's child-pair records, 64 bytes each: left child's
                                        box (6 floats), right child's box, left ref, right ref (internal:
                                        record index; leaf: 0x80000000 | first sorted triangle), 0, 0 --
                                        the sibling pairs of the reference's LEFT_OFFSET array
                                        (lbvh.cpp:492-729) in the LR tree's numbering                       */
int hrt_geom_export(const hrt_scene* scene, uint32_t geomId, int what, void* dst, uint64_t capacityBytes,
                    uint64_t* sizeBytes);

/* Page-locked host memory for the host-pointer queries (copies from it run at
 * full link speed).  No reference counterpart: the reference is host-only. */
int hrt_host_alloc(uint64_t bytes, void** out);
int hrt_host_free(void* p);

/* Stable sort of (Morton code, triangle id) pairs by code -- the LBVH build's
 * radix sort -- that allocates nothing.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: host applications whose device
 * memory is owned by another allocator that reserves it up front (a renderer
 * or engine with its own device heap, a process under a hard memory quota),
 * and latency-bound paths that cannot take an allocation's implicit
 * synchronisation.  keys and vals are device arrays of n entries (input and
 * output, sorted in place); all scratch comes from one fixed device array that
 * the library holds on every GPU that loads it (about 2.4 MB) until the process
 * exits.  n above HRT_NOALLOC_MAX_PAIRS is rejected with HRT_ERR_CAPACITY.
 *
 * Runs on the calling thread's current device and on `stream`, and returns
 * after the stream has finished the sort (HRT_ERR_TIMEOUT if a device wait gave
 * up).  The first call on a device resolves the scratch array's device address
 * (cudaGetSymbolAddress) and keeps it; make that first call before any stream
 * capture begins, and do not use the function on a device after
 * cudaDeviceReset.  Every call shares the one array, which keeps the last
 * call's contents (the call clears what must start at zero), so calls whose
 * work overlaps on the GPU race with each other: serialise them (one stream,
 * or wait between calls). */
#define HRT_NOALLOC_MAX_PAIRS (1u << 18)
int hrt_sort_morton_pairs_noalloc(uint32_t* keys, uint32_t* vals, uint64_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HRT_H */
