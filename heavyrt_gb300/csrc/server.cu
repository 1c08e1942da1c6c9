// Serving loop (include/hrt.h, hrt_server_*): scenes resident in HBM, builds
// on arrival, admission against a device-memory budget, continuous batching of
// ray requests with overlapping in-flight batches.
//
// Threads:
//   builder     builds queued scenes one at a time on its own stream (the LBVH
//               build of hrt_add_geom_triangles3f), writes the scene's entry
//               of the device scene table, then marks it ready; frees the
//               geometry of evicted / removed scenes;
//   dispatcher  whenever a batch slot is free, takes the queued requests whose
//               scenes are ready (arrival order, up to the slot's capacity),
//               and issues them on the slot's stream: ray copies in, one
//               segmented traversal per query kind over the scene table, result
//               copies out, then a host callback;
//   callback    (CUDA's host-function thread) marks the slot's requests done
//               and frees the slot.
// No CUDA call is made while the server lock is held, and the callback makes
// none, so the callback can never wait on a thread that waits on the GPU.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <unordered_map>

#include "hrt_internal.cuh"

using namespace hrt;
using namespace hrt::api;

namespace
{

constexpr uint32_t kSlotBits = 16;  // scene id = generation << 16 | table slot
constexpr uint32_t kSlotMask = (1u << kSlotBits) - 1u;

struct Request
{
  uint64_t         ticket = 0;
  uint32_t         scene = 0;  // table slot
  int              kind = 0;
  const float*     rays = nullptr;
  uint64_t         n = 0;
  void*            out = nullptr;
  bool             done = false;
  hrt_request_info info{};
};

struct SceneRec
{
  int                   state = HRT_SCENE_EVICTED;  // a free table slot reads as evicted
  uint32_t              gen = 0;
  bool                  evictable = true;
  uint32_t              refs = 0;      // queued + in-flight requests
  uint64_t              lastUse = 0;
  uint64_t              reserved = 0;  // bytes held against the budget
  Geom                  geom;
  InstanceDesc          desc{};            // host copy of the scene's table entry (valid once ready)
  void*                 dVerts = nullptr;  // inputs of a pending build, copied to the device
  uint32_t*             dIdx = nullptr;
  uint64_t              nIdx = 0;
  uint64_t              nVert = 0, stride = 0;
};

struct Slot;

}  // namespace

struct hrt_server
{
  hrt_context*            ctx = nullptr;  // the caller's context (device)
  hrt_context             bctx;           // builder's stream
  cudaStream_t            stageStream = nullptr;  // copies of new scenes' inputs
  hrt_scene               proto;          // layout / merge options for builds
  hrt_server_config       cfg{};
  TraceConfig             trace[2];     // segmented batches
  TraceConfig             traceOne[2];  // batches of one request (single-instance kernels)
  InstanceDesc*           dTable = nullptr;
  std::vector<SceneRec>   scenes;
  std::vector<uint32_t>   freeSlots;
  std::vector<Slot*>      slots;
  std::deque<Request*>    queue;
  std::unordered_map<uint64_t, Request*> tickets;
  std::deque<uint32_t>    buildQueue;
  std::vector<Geom>       toFree;
  std::mutex              mu;
  std::condition_variable cvDispatch, cvDone, cvBuild;
  std::thread             dispatcher, builder;
  bool                    stop = false;
  uint64_t                nextTicket = 1, useClock = 0;
  uint32_t                nextBatch = 0;
  uint64_t                resident = 0, peakResident = 0;
  hrt_server_stats        stats{};
  std::chrono::steady_clock::time_point t0;

  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace
{

struct Slot
{
  hrt_server*           server = nullptr;
  cudaStream_t          stream = nullptr;
  float4*               rays = nullptr;   // 2 float4 per ray: nearest rays, then any rays
  hrt_hit*              hits = nullptr;
  uint8_t*              any = nullptr;
  uint32_t*             dIdx = nullptr;   // [kind][offsets maxReq+1 | segments maxReq]
  uint32_t*             hIdx = nullptr;   // pinned staging of dIdx
  uint32_t*             dErr = nullptr;   // error word (8 words)
  uint32_t*             hErr = nullptr;   // pinned copy
  unsigned int*         counters = nullptr;
  bool                  busy = false;
  uint32_t              batch = 0;
  std::vector<Request*> reqs;
  InstanceDesc          one{};  // the scene of a batch of one request (copied under the server lock)
};

uint64_t estimate_scene_bytes(uint64_t nTris, uint64_t nVert, int layout)
{
  const uint64_t N = nTris ? nTris : 1;
  uint64_t b = 16 * nVert + N * (4 * 5 + sizeof(TriRec) + 12) + (2 * N) * (sizeof(BVHNode32) + 4) +
               sizeof(BuildParams);
  if (layout == HRT_LAYOUT_BVH2) b += N * sizeof(PairRec);
  else b += N * (layout == HRT_LAYOUT_BVH4_F32 ? sizeof(Node4F32) : sizeof(Node4F16));
  // transient build arrays (ping-pong, parents, visit counters, sort scratch)
  b += N * 4 * 6 + radix_sort_scratch_bytes((uint32_t)N) + 4 * 1024 * 32;
  // the staged copy of the inputs (16-byte vertices, indices) held until the build
  b += 16 * nVert + 12 * (uint64_t)nTris;
  return b;
}

size_t slot_bytes(const hrt_server_config& c)
{
  return c.slotRays * (32 + sizeof(hrt_hit) + 1) + 2 * sizeof(uint32_t) * (2 * (size_t)c.maxBatchRequests + 1) + 64;
}

void finish(hrt_server* S, Request* r, int status)
{
  r->info.status = status;
  r->info.tDone = S->now();
  r->done = true;
  if (status != HRT_OK) S->stats.failed++;
}

// CUDA host-function callback at the end of a slot's stream work.
void CUDART_CB on_slot_done(void* p)
{
  Slot* sl = static_cast<Slot*>(p);
  hrt_server* S = sl->server;
  {
    std::lock_guard<std::mutex> g(S->mu);
    const uint32_t err = sl->hErr[0];
    const int st = err ? HRT_ERR_DEVICE_CHECK : HRT_OK;
    for (Request* r : sl->reqs)
    {
      finish(S, r, st);
      S->scenes[r->scene].refs--;
      if (st == HRT_OK)
      {
        S->stats.requests++;
        S->stats.rays += r->n;
      }
    }
    sl->reqs.clear();
    sl->busy = false;
  }
  S->cvDone.notify_all();
  S->cvDispatch.notify_one();
}

// Issues one batch on a slot (outside the lock).  Returns a CUDA error, in
// which case nothing was queued behind the last successful call and the caller
// fails the batch.
cudaError_t issue(hrt_server* S, Slot* sl)
{
  const uint32_t maxReq = S->cfg.maxBatchRequests;
  // A batch of one request whose rays are page-locked (and 16-byte aligned)
  // reads them in place over the host link (no copy in); its any-hit flags are
  // written in place too when the output is page-locked.
  const Request* only = sl->reqs.size() == 1 ? sl->reqs[0] : nullptr;
  const float4* inPlaceRays =
      only && aligned_to(only->rays, 16) ? static_cast<const float4*>(mapped_host(only->rays)) : nullptr;
  void* inPlaceOut =
      only && (only->kind == 1 || aligned_to(only->out, 16)) ? mapped_host(only->out) : nullptr;
  if (only && sl->one.valid)
  {
    // One request against one scene of one untransformed geometry: the
    // single-instance kernels (fewer registers, no segment search), rays read
    // in place when page-locked, results written in place when page-locked
    // (nearest hits by the one-thread-per-ray kernel, whose warps write 32
    // consecutive hits at once); the same results as the segmented launch.
    cudaStream_t st = sl->stream;
    cudaError_t e = cudaMemsetAsync(sl->dErr, 0, 8 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    const int k = only->kind;
    if (!inPlaceRays)
    {
      e = cudaMemcpyAsync(sl->rays, only->rays, 32 * only->n, cudaMemcpyHostToDevice, st);
      if (e != cudaSuccess) return e;
    }
    TraceArgs a;
    a.rays = inPlaceRays ? inPlaceRays : sl->rays;
    a.n = only->n;
    a.inst = S->dTable;
    a.nInst = S->cfg.maxScenes;
    a.hits = inPlaceOut ? inPlaceOut : (k == 0 ? static_cast<void*>(sl->hits) : static_cast<void*>(sl->any));
    a.counters = nullptr;
    a.errorWord = sl->dErr;
    a.rayCounter = sl->counters + k;
    a.one = &sl->one;
    TraceConfig c = S->traceOne[k];
    if (k == 0 && inPlaceOut) c.persistent = 0;
    e = hrt::trace(a, k, 0, S->cfg.layout, c, S->ctx->numSMs, st);
    if (e != cudaSuccess) return e;
    if (!inPlaceOut)
    {
      e = k == 0 ? cudaMemcpyAsync(only->out, sl->hits, sizeof(hrt_hit) * only->n, cudaMemcpyDeviceToHost, st)
                 : cudaMemcpyAsync(only->out, sl->any, only->n, cudaMemcpyDeviceToHost, st);
      if (e != cudaSuccess) return e;
    }
    e = cudaMemcpyAsync(sl->hErr, sl->dErr, 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    return cudaLaunchHostFunc(st, on_slot_done, sl);
  }
  if (only && only->kind == 0) inPlaceOut = nullptr;  // the segmented path copies nearest hits out
  uint32_t* hOff[2] = {sl->hIdx, sl->hIdx + (2 * maxReq + 1)};
  uint32_t* dOff[2] = {sl->dIdx, sl->dIdx + (2 * maxReq + 1)};
  uint32_t cnt[2] = {0, 0};
  uint64_t total[2] = {0, 0};
  for (const Request* r : sl->reqs) total[r->kind] += r->n;
  hOff[0][0] = hOff[1][0] = 0;
  cudaStream_t st = sl->stream;
  cudaError_t e = cudaSuccess;
  for (const Request* r : sl->reqs)
  {
    const int k = r->kind;
    const uint64_t base = (k == 0 ? 0 : total[0]) + hOff[k][cnt[k]];
    if (!inPlaceRays)
    {
      e = cudaMemcpyAsync(sl->rays + 2 * base, r->rays, 32 * r->n, cudaMemcpyHostToDevice, st);
      if (e != cudaSuccess) return e;
    }
    hOff[k][maxReq + 1 + cnt[k]] = r->scene;  // segment -> scene table slot
    hOff[k][cnt[k] + 1] = hOff[k][cnt[k]] + (uint32_t)r->n;
    cnt[k]++;
  }
  e = cudaMemcpyAsync(sl->dIdx, sl->hIdx, sizeof(uint32_t) * 2 * (2 * maxReq + 1), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(sl->dErr, 0, 8 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  for (int k = 0; k < 2; k++)
  {
    if (!cnt[k]) continue;
    TraceArgs a;
    a.rays = inPlaceRays ? inPlaceRays : sl->rays + 2 * (k == 0 ? 0 : total[0]);
    a.n = total[k];
    a.inst = S->dTable;
    a.nInst = S->cfg.maxScenes;
    a.hits = k == 0 ? static_cast<void*>(sl->hits) : (inPlaceOut ? inPlaceOut : static_cast<void*>(sl->any));
    a.counters = nullptr;
    a.errorWord = sl->dErr;
    a.rayCounter = sl->counters + k;
    a.rayOffsets = dOff[k];
    a.segInst = dOff[k] + maxReq + 1;
    a.nSeg = cnt[k];
    e = hrt::trace(a, k, 0, S->cfg.layout, S->trace[k], S->ctx->numSMs, st);
    if (e != cudaSuccess) return e;
  }
  uint32_t pos[2] = {0, 0};
  for (const Request* r : sl->reqs)
  {
    const int k = r->kind;
    if (k == 0) e = cudaMemcpyAsync(r->out, sl->hits + pos[0], sizeof(hrt_hit) * r->n, cudaMemcpyDeviceToHost, st);
    else if (!inPlaceOut) e = cudaMemcpyAsync(r->out, sl->any + pos[1], r->n, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    pos[k] += (uint32_t)r->n;
  }
  e = cudaMemcpyAsync(sl->hErr, sl->dErr, 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  return cudaLaunchHostFunc(st, on_slot_done, sl);
}

void dispatcher_main(hrt_server* S)
{
  cudaSetDevice(S->ctx->device);
  std::unique_lock<std::mutex> lk(S->mu);
  while (true)
  {
    Slot* free = nullptr;
    for (Slot* sl : S->slots)
      if (!sl->busy)
      {
        free = sl;
        break;
      }
    // requests of failed / removed scenes complete at once
    bool ready = false;
    for (auto it = S->queue.begin(); it != S->queue.end();)
    {
      const int state = S->scenes[(*it)->scene].state;
      if (state == HRT_SCENE_FAILED || state == HRT_SCENE_EVICTED)
      {
        finish(S, *it, HRT_ERR_STATE);
        S->scenes[(*it)->scene].refs--;
        it = S->queue.erase(it);
        S->cvDone.notify_all();
        continue;
      }
      ready = ready || state == HRT_SCENE_READY;
      ++it;
    }
    if (S->stop && S->queue.empty()) break;
    if (!free || !ready)
    {
      S->cvDispatch.wait(lk);
      continue;
    }
    // continuous batching: everything queued and ready that fits, in arrival order
    uint64_t rays = 0;
    for (auto it = S->queue.begin(); it != S->queue.end();)
    {
      Request* r = *it;
      if (S->scenes[r->scene].state != HRT_SCENE_READY)
      {
        ++it;
        continue;
      }
      if (rays + r->n > S->cfg.slotRays || free->reqs.size() >= S->cfg.maxBatchRequests) break;
      rays += r->n;
      free->reqs.push_back(r);
      S->scenes[r->scene].lastUse = ++S->useClock;
      it = S->queue.erase(it);
    }
    if (free->reqs.empty()) continue;
    free->one = InstanceDesc{};
    if (free->reqs.size() == 1)
    {
      const InstanceDesc& d = S->scenes[free->reqs[0]->scene].desc;
      if (d.valid && d.identity) free->one = d;
    }
    free->busy = true;
    free->batch = S->nextBatch++;
    const double t = S->now();
    for (Request* r : free->reqs)
    {
      r->info.tStart = t;
      r->info.batch = free->batch;
      r->info.batchRequests = (uint32_t)free->reqs.size();
      r->info.batchRays = rays;
    }
    S->stats.batches++;
    lk.unlock();
    const cudaError_t e = issue(S, free);
    lk.lock();
    if (e != cudaSuccess)
    {
      // nothing more arrives on this slot's stream for this batch: wait for
      // what was queued, then fail the batch
      lk.unlock();
      cudaStreamSynchronize(free->stream);
      lk.lock();
      for (Request* r : free->reqs)
      {
        finish(S, r, HRT_ERR_CUDA);
        S->scenes[r->scene].refs--;
      }
      free->reqs.clear();
      free->busy = false;
      S->cvDone.notify_all();
    }
  }
}

void builder_main(hrt_server* S)
{
  cudaSetDevice(S->ctx->device);
  std::unique_lock<std::mutex> lk(S->mu);
  while (true)
  {
    S->cvBuild.wait(lk, [&] { return S->stop || !S->buildQueue.empty() || !S->toFree.empty(); });
    if (!S->toFree.empty())
    {
      std::vector<Geom> frees;
      frees.swap(S->toFree);
      lk.unlock();
      cudaStreamSynchronize(S->bctx.stream);
      for (Geom& g : frees) free_geom(g);
      lk.lock();
      continue;
    }
    if (S->buildQueue.empty())
    {
      if (S->stop) break;
      continue;
    }
    const uint32_t slot = S->buildQueue.front();
    S->buildQueue.pop_front();
    SceneRec& sc = S->scenes[slot];
    void* dVerts = sc.dVerts;
    uint32_t* dIdx = sc.dIdx;
    sc.dVerts = nullptr;
    sc.dIdx = nullptr;
    const uint64_t nVert = sc.nVert, nIdx = sc.nIdx, stride = sc.stride;
    lk.unlock();
    Geom g;
    int st = build_geometry(&S->proto, g, reinterpret_cast<const float*>(dVerts), nVert, dIdx, nIdx, stride,
                            S->cfg.layout);
    // the staged inputs are released in stream order, after the build's copies
    if (dVerts) cudaFreeAsync(dVerts, S->bctx.stream);
    if (dIdx) cudaFreeAsync(dIdx, S->bctx.stream);
    InstanceDesc d;
    if (st == HRT_OK)
    {
      make_instance_desc(g, slot, slot, nullptr, d);
      if (cudaMemcpyAsync(S->dTable + slot, &d, sizeof(d), cudaMemcpyHostToDevice, S->bctx.stream) != cudaSuccess ||
          cudaStreamSynchronize(S->bctx.stream) != cudaSuccess)
        st = HRT_ERR_CUDA;
    }
    if (st != HRT_OK)
    {
      cudaStreamSynchronize(S->bctx.stream);
      free_geom(g);
      fail(S->ctx, st, "scene build failed: " + S->bctx.lastError);
    }
    lk.lock();
    S->resident -= sc.reserved;
    if (st == HRT_OK)
    {
      sc.geom = g;
      sc.desc = d;
      sc.reserved = g.bytes;
      sc.state = HRT_SCENE_READY;
      S->resident += g.bytes;
      S->stats.builds++;
    }
    else
    {
      sc.reserved = 0;
      sc.state = HRT_SCENE_FAILED;
    }
    S->peakResident = std::max(S->peakResident, S->resident);
    S->cvDispatch.notify_one();
    S->cvDone.notify_all();
  }
}

// Frees the table slot of a ready scene (lock held); its geometry goes to the
// builder, which frees it.
void release_scene(hrt_server* S, uint32_t slot)
{
  SceneRec& sc = S->scenes[slot];
  S->resident -= sc.reserved;
  sc.reserved = 0;
  if (sc.state == HRT_SCENE_READY) S->toFree.push_back(sc.geom);
  sc.geom = Geom();
  sc.state = HRT_SCENE_EVICTED;
  sc.gen = (sc.gen + 1) & 0xFFFFu;
  S->freeSlots.push_back(slot);
  S->cvBuild.notify_one();
}

bool decode(hrt_server* S, uint32_t id, uint32_t& slot)
{
  slot = id & kSlotMask;
  return slot < S->scenes.size() && S->scenes[slot].gen == (id >> kSlotBits);
}

void destroy_slots(hrt_server* S)
{
  for (Slot* sl : S->slots)
  {
    if (sl->stream) cudaStreamSynchronize(sl->stream);
    if (sl->stream) cudaStreamDestroy(sl->stream);
    cudaFree(sl->rays);
    cudaFree(sl->hits);
    cudaFree(sl->any);
    cudaFree(sl->dIdx);
    cudaFree(sl->dErr);
    cudaFree(sl->counters);
    if (sl->hIdx) cudaFreeHost(sl->hIdx);
    if (sl->hErr) cudaFreeHost(sl->hErr);
    delete sl;
  }
  S->slots.clear();
}

}  // namespace

extern "C" {

int hrt_server_create(hrt_context* ctx, const hrt_server_config* config, hrt_server** out)
{
  if (!ctx || !out) return HRT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  hrt_server_config c = config ? *config : hrt_server_config{};
  if (c.memoryBudget == 0) c.memoryBudget = 150000000000ull;
  if (c.slotRays == 0) c.slotRays = 8u << 20;
  if (c.slots == 0) c.slots = 3;
  if (c.maxScenes == 0) c.maxScenes = 4096;
  if (c.maxBatchRequests == 0) c.maxBatchRequests = 1024;
  if (c.maxScenes > (1u << kSlotBits) || c.slots > 16 || c.slotRays > 0xFFFFFFFFull ||
      c.layout < HRT_LAYOUT_BVH2 || c.layout > HRT_LAYOUT_BVH4_Q8 || c.bvh4Merge < 0 || c.bvh4Merge > 64 ||
      (c.mortonFrame != HRT_MORTON_PER_AXIS && c.mortonFrame != HRT_MORTON_CUBIC) ||
      (c.bvh4Collapse != HRT_BVH4_COLLAPSE_EVEN_DEPTH && c.bvh4Collapse != HRT_BVH4_COLLAPSE_LARGEST_FIRST))
    return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "server configuration out of range");
  const uint64_t staging = (uint64_t)c.slots * slot_bytes(c);
  if (staging + sizeof(InstanceDesc) * (uint64_t)c.maxScenes > c.memoryBudget)
    return fail(ctx, HRT_ERR_CAPACITY, "memory budget smaller than the batch slots");
  cudaSetDevice(ctx->device);
  hrt_server* S = new hrt_server();
  S->ctx = ctx;
  S->cfg = c;
  S->bctx.device = ctx->device;
  S->bctx.numSMs = ctx->numSMs;
  S->proto.ctx = &S->bctx;
  S->proto.layout = c.layout;
  S->proto.bvh4Merge = c.bvh4Merge;
  S->proto.mortonFrame = c.mortonFrame;
  S->proto.bvh4Collapse = c.bvh4Collapse;
  for (int k = 0; k < 2; k++)
  {
    S->trace[k].threadsPerBlock = 256;  // segmented batches: fastest shape of the batched-scene sweep
    S->trace[k].persistent = 1;
    S->trace[k].stepsPerRefill = 16;
    S->trace[k].refillLanes = 8;
  }
  // single requests: the single-instance kernels' shapes of the RTAO frame's
  // sweep (nearest hits written in place switch to one thread per ray)
  S->traceOne[0].threadsPerBlock = 64;
  S->traceOne[0].persistent = 0;
  S->traceOne[1].threadsPerBlock = 128;
  S->traceOne[1].persistent = 1;
  S->traceOne[1].stepsPerRefill = 8;
  S->traceOne[1].refillLanes = 8;
  auto bail = [&](cudaError_t e, const char* what) {
    destroy_slots(S);
    if (S->dTable) cudaFree(S->dTable);
    if (S->bctx.stream) cudaStreamDestroy(S->bctx.stream);
    if (S->stageStream) cudaStreamDestroy(S->stageStream);
    delete S;
    return cuda_fail(ctx, e, what);
  };
  // ray batches run at the highest stream priority, builds and uploads at the
  // lowest: the block scheduler then serves a batch's blocks first whenever
  // both wait for SMs, so builds on arrival delay queries as little as possible
  int leastPriority = 0, greatestPriority = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&leastPriority, &greatestPriority);
  if (e != cudaSuccess) return bail(e, "stream priorities");
  e = cudaStreamCreateWithPriority(&S->bctx.stream, cudaStreamNonBlocking, leastPriority);
  if (e != cudaSuccess) return bail(e, "builder stream");
  e = cudaStreamCreateWithPriority(&S->stageStream, cudaStreamNonBlocking, leastPriority);
  if (e != cudaSuccess) return bail(e, "staging stream");
  e = cudaMalloc((void**)&S->dTable, sizeof(InstanceDesc) * c.maxScenes);
  if (e != cudaSuccess) return bail(e, "scene table");
  e = cudaMemset(S->dTable, 0, sizeof(InstanceDesc) * c.maxScenes);  // valid = 0 everywhere
  if (e != cudaSuccess) return bail(e, "scene table");
  for (uint32_t i = 0; i < c.slots; i++)
  {
    Slot* sl = new Slot();
    S->slots.push_back(sl);
    sl->server = S;
    const size_t idxWords = 2 * (2 * (size_t)c.maxBatchRequests + 1);
    if ((e = cudaStreamCreateWithPriority(&sl->stream, cudaStreamNonBlocking, greatestPriority)) != cudaSuccess ||
        (e = cudaMalloc((void**)&sl->rays, 32 * c.slotRays)) != cudaSuccess ||
        (e = cudaMalloc((void**)&sl->hits, sizeof(hrt_hit) * c.slotRays)) != cudaSuccess ||
        (e = cudaMalloc((void**)&sl->any, c.slotRays)) != cudaSuccess ||
        (e = cudaMalloc((void**)&sl->dIdx, sizeof(uint32_t) * idxWords)) != cudaSuccess ||
        (e = cudaMalloc((void**)&sl->dErr, 8 * sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMalloc((void**)&sl->counters, 2 * sizeof(unsigned int))) != cudaSuccess ||
        (e = cudaMallocHost((void**)&sl->hIdx, sizeof(uint32_t) * idxWords)) != cudaSuccess ||
        (e = cudaMallocHost((void**)&sl->hErr, 8 * sizeof(uint32_t))) != cudaSuccess)
      return bail(e, "batch slot");
  }
  S->resident = staging + sizeof(InstanceDesc) * (uint64_t)c.maxScenes;
  S->peakResident = S->resident;
  S->scenes.resize(c.maxScenes);
  for (uint32_t i = c.maxScenes; i > 0; i--) S->freeSlots.push_back(i - 1);
  S->t0 = std::chrono::steady_clock::now();
  S->dispatcher = std::thread(dispatcher_main, S);
  S->builder = std::thread(builder_main, S);
  *out = S;
  return HRT_OK;
}

int hrt_server_destroy(hrt_server* S)
{
  if (!S) return HRT_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stop = true;
  }
  S->cvDispatch.notify_all();
  S->cvBuild.notify_all();
  S->builder.join();  // finishes queued builds first, so queued requests can run
  {
    std::lock_guard<std::mutex> g(S->mu);
  }
  S->cvDispatch.notify_all();
  S->dispatcher.join();
  cudaSetDevice(S->ctx->device);
  destroy_slots(S);
  for (SceneRec& sc : S->scenes)
    if (sc.state == HRT_SCENE_READY) free_geom(sc.geom);
  for (Geom& g : S->toFree) free_geom(g);
  for (auto& kv : S->tickets) delete kv.second;
  cudaFree(S->dTable);
  cudaStreamSynchronize(S->stageStream);
  cudaStreamDestroy(S->stageStream);
  cudaStreamDestroy(S->bctx.stream);
  delete S;
  return HRT_OK;
}

int hrt_server_add_scene(hrt_server* S, const float* vpos, uint64_t nVert, const uint32_t* idx, uint64_t nIdx,
                         uint64_t vByteStride, int evictable, uint32_t* sceneId)
{
  if (!S || !sceneId) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = S->ctx;
  if (vByteStride == 0) vByteStride = 12;
  if (vByteStride < 12 || vByteStride % 4 != 0)
    return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "vByteStride must be >= 12 and a multiple of 4");
  if (nIdx % 3 != 0) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "index count is not a multiple of 3");
  if ((nVert && !vpos) || (nIdx && !idx)) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "null vertex or index pointer");
  if (nIdx / 3 > HRT_MAX_TRIS_PER_GEOM) return fail(ctx, HRT_ERR_CAPACITY, "more than 2^24-1 triangles in one scene");
  if (nVert > 0xFFFFFFFFull) return fail(ctx, HRT_ERR_CAPACITY, "more than 2^32-1 vertices in one scene");
  const uint64_t need =
      estimate_scene_bytes(nIdx / 3, nVert, S->cfg.layout) + (vByteStride > 16 ? (vByteStride - 16) * nVert : 0);
  // Copy the inputs to the device before taking the lock (the caller owns
  // them only for the call): one copy, at full link speed from page-locked
  // memory; the builder reads them from there.
  cudaSetDevice(ctx->device);
  void* dV = nullptr;
  uint32_t* dI = nullptr;
  auto unstage = [&]() {
    if (dV) cudaFreeAsync(dV, S->stageStream);
    if (dI) cudaFreeAsync(dI, S->stageStream);
    dV = nullptr;
    dI = nullptr;
  };
  {
    cudaError_t e = cudaSuccess;
    if (nVert) e = cudaMallocAsync(&dV, vByteStride * nVert, S->stageStream);
    if (e == cudaSuccess && nIdx) e = cudaMallocAsync((void**)&dI, 4 * nIdx, S->stageStream);
    if (e == cudaSuccess && nVert)
      e = cudaMemcpyAsync(dV, vpos, vByteStride * nVert, cudaMemcpyDefault, S->stageStream);
    if (e == cudaSuccess && nIdx) e = cudaMemcpyAsync(dI, idx, 4 * nIdx, cudaMemcpyDefault, S->stageStream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S->stageStream);
    if (e != cudaSuccess)
    {
      unstage();
      return cuda_fail(ctx, e, "staging a new scene's inputs");
    }
  }
  std::unique_lock<std::mutex> g(S->mu);
  auto reject = [&](int status, const char* msg) {
    g.unlock();
    unstage();
    return fail(ctx, status, msg);
  };
  if (S->stop) return reject(HRT_ERR_STATE, "server is shutting down");
  // admission: evict idle evictable scenes, least recently used first - and
  // only when evicting all of them would make room
  uint64_t freeable = 0;
  for (const SceneRec& sc : S->scenes)
    if (sc.state == HRT_SCENE_READY && sc.evictable && sc.refs == 0) freeable += sc.reserved;
  if (S->resident - freeable + need > S->cfg.memoryBudget)
    return reject(HRT_ERR_OUT_OF_MEMORY, "scene does not fit the memory budget");
  while (S->resident + need > S->cfg.memoryBudget)
  {
    int64_t victim = -1;
    for (uint32_t i = 0; i < S->scenes.size(); i++)
    {
      const SceneRec& sc = S->scenes[i];
      if (sc.state == HRT_SCENE_READY && sc.evictable && sc.refs == 0 &&
          (victim < 0 || sc.lastUse < S->scenes[victim].lastUse))
        victim = i;
    }
    if (victim < 0) return reject(HRT_ERR_OUT_OF_MEMORY, "scene does not fit the memory budget");
    release_scene(S, (uint32_t)victim);
    S->stats.evictions++;
  }
  if (S->freeSlots.empty()) return reject(HRT_ERR_CAPACITY, "scene table full");
  const uint32_t slot = S->freeSlots.back();
  S->freeSlots.pop_back();
  SceneRec& sc = S->scenes[slot];
  sc.state = HRT_SCENE_BUILDING;
  sc.evictable = evictable != 0;
  sc.refs = 0;
  sc.lastUse = ++S->useClock;
  sc.reserved = need;
  sc.dVerts = dV;
  sc.dIdx = dI;
  sc.nIdx = nIdx;
  sc.nVert = nVert;
  sc.stride = vByteStride;
  S->resident += need;
  S->peakResident = std::max(S->peakResident, S->resident);
  S->buildQueue.push_back(slot);
  *sceneId = (sc.gen << kSlotBits) | slot;
  S->cvBuild.notify_one();
  return HRT_OK;
}

int hrt_server_scene_state(hrt_server* S, uint32_t sceneId, double timeoutSeconds, int* state)
{
  if (!S || !state) return HRT_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(S->mu);
  uint32_t slot;
  if (!decode(S, sceneId, slot))
  {
    *state = HRT_SCENE_EVICTED;
    return HRT_OK;
  }
  auto settled = [&] { return S->scenes[slot].state != HRT_SCENE_BUILDING || S->scenes[slot].gen != (sceneId >> kSlotBits); };
  if (timeoutSeconds > 0)
    S->cvDone.wait_for(lk, std::chrono::duration<double>(timeoutSeconds), settled);
  else if (timeoutSeconds < 0)
    S->cvDone.wait(lk, settled);
  *state = S->scenes[slot].gen == (sceneId >> kSlotBits) ? S->scenes[slot].state : HRT_SCENE_EVICTED;
  return HRT_OK;
}

int hrt_server_remove_scene(hrt_server* S, uint32_t sceneId)
{
  if (!S) return HRT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(S->mu);
  uint32_t slot;
  if (!decode(S, sceneId, slot) || S->scenes[slot].state == HRT_SCENE_EVICTED)
    return fail(S->ctx, HRT_ERR_INVALID_ARGUMENT, "unknown scene id");
  SceneRec& sc = S->scenes[slot];
  if (sc.state == HRT_SCENE_BUILDING || sc.refs > 0)
    return fail(S->ctx, HRT_ERR_STATE, "scene is being built or has requests in flight");
  release_scene(S, slot);
  return HRT_OK;
}

int hrt_server_submit(hrt_server* S, uint32_t sceneId, int kind, const float* rays, uint64_t n, void* out,
                      uint64_t* ticket)
{
  if (!S || !ticket) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = S->ctx;
  if (kind != 0 && kind != 1) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "unknown query kind");
  if (n && (!rays || !out)) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "null ray or output pointer");
  if (n > S->cfg.slotRays) return fail(ctx, HRT_ERR_CAPACITY, "request larger than a batch slot");
  std::unique_lock<std::mutex> lk(S->mu);
  uint32_t slot;
  if (!decode(S, sceneId, slot)) return fail(ctx, HRT_ERR_STATE, "scene was evicted or removed");
  SceneRec& sc = S->scenes[slot];
  if (sc.state == HRT_SCENE_FAILED || sc.state == HRT_SCENE_EVICTED)
    return fail(ctx, HRT_ERR_STATE, "scene failed to build, was evicted or removed");
  if (S->stop) return fail(ctx, HRT_ERR_STATE, "server is shutting down");
  Request* r = new Request();
  r->ticket = S->nextTicket++;
  r->scene = slot;
  r->kind = kind;
  r->rays = rays;
  r->n = n;
  r->out = out;
  r->info.tSubmit = S->now();
  S->tickets[r->ticket] = r;
  *ticket = r->ticket;
  if (n == 0)
  {
    finish(S, r, HRT_OK);
    return HRT_OK;
  }
  sc.refs++;
  S->queue.push_back(r);
  lk.unlock();
  S->cvDispatch.notify_one();
  return HRT_OK;
}

int hrt_server_wait(hrt_server* S, uint64_t ticket, double timeoutSeconds, hrt_request_info* info)
{
  if (!S) return HRT_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->tickets.find(ticket);
  if (it == S->tickets.end()) return fail(S->ctx, HRT_ERR_INVALID_ARGUMENT, "unknown ticket");
  Request* r = it->second;
  if (timeoutSeconds < 0)
    S->cvDone.wait(lk, [&] { return r->done; });
  else if (!r->done)
    S->cvDone.wait_for(lk, std::chrono::duration<double>(timeoutSeconds), [&] { return r->done; });
  if (!r->done) return HRT_ERR_TIMEOUT;
  if (info) *info = r->info;
  const int st = r->info.status;
  S->tickets.erase(it);
  delete r;
  return st;
}

int hrt_server_get_stats(hrt_server* S, hrt_server_stats* out)
{
  if (!S || !out) return HRT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(S->mu);
  *out = S->stats;
  out->residentBytes = S->resident;
  out->peakResidentBytes = S->peakResident;
  out->queued = (uint32_t)S->queue.size();
  uint32_t nres = 0;
  for (const SceneRec& sc : S->scenes) nres += (sc.state == HRT_SCENE_READY);
  out->scenesResident = nres;
  return HRT_OK;
}

int hrt_server_scene_bytes(const hrt_server* S, uint64_t nVert, uint64_t nTris, uint64_t* bytes)
{
  if (!S || !bytes) return HRT_ERR_INVALID_ARGUMENT;
  *bytes = estimate_scene_bytes(nTris, nVert, S->cfg.layout);
  return HRT_OK;
}

}  // extern "C"
