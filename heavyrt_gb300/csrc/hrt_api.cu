// C ABI of the engine (include/hrt.h): contexts, scenes, geometry builds,
// instances and batched queries.  Host-side bookkeeping mirrors
// BVH2CommonRT's (core/BVH2CommonRT.h:70-87, core/BVH2CommonRT_host.cpp); every
// array it keeps lives in device memory.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "hrt_internal.cuh"

using namespace hrt;
using namespace hrt::api;



namespace hrt
{
namespace api
{

int fail(hrt_context* ctx, int status, const std::string& msg)
{
  if (ctx)
  {
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->lastError = msg;
  }
  return status;
}

int cuda_fail(hrt_context* ctx, cudaError_t e, const char* what)
{
  const int st = (e == cudaErrorMemoryAllocation) ? HRT_ERR_OUT_OF_MEMORY : HRT_ERR_CUDA;
  return fail(ctx, st, std::string(what) + ": " + cudaGetErrorString(e));
}


void free_geom(Geom& g)
{
  if (!g.shared)
  {
    void* ptrs[] = {g.verts, g.keys, g.vals, g.keysUnsorted, g.compressed, g.runStarts, g.lr,
                    g.lrCount, g.recs, g.tris, g.sortedIdx, g.params, g.nodes4};
    bool any = false;
    for (void* p : ptrs) any = any || p != nullptr;
    // the arrays come from the stream-ordered pool, whose cudaFree does not
    // wait: finish every query that may still read them first
    if (any) cudaDeviceSynchronize();
    for (void* p : ptrs)
      if (p) cudaFree(p);
  }
  g = Geom();
}

// A geometry array from the device's stream-ordered pool (no implicit
// synchronisation, blocks reused from earlier builds); free_geom waits for the
// device before it frees, so no query in flight loses it.
template <typename T> cudaError_t dalloc(T** p, size_t count, uint64_t* bytes, cudaStream_t st)
{
  const size_t b = sizeof(T) * (count ? count : 1);
  if (bytes) *bytes += b;
  return cudaMallocAsync((void**)p, b, st);
}

__global__ void k_pack_verts(const uint8_t* __restrict__ raw, uint64_t n, uint64_t stride, float4* __restrict__ out)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    const float* p = reinterpret_cast<const float*>(raw + i * stride);
    out[i] = make_float4(p[0], p[1], p[2], 1.0f);
  }
}

// Inverse of a column-major 4x4 through the adjugate, in float, the same
// evaluation as the reference checker's LiteMath stand-in.
void inverse4x4(const float* mc, float* inv12)
{
  float a[4][4];
  for (int r = 0; r < 4; r++)
    for (int c = 0; c < 4; c++) a[r][c] = mc[c * 4 + r];
  auto minor3 = [&](int skipR, int skipC) {
    float s[3][3];
    int rr = 0;
    for (int r = 0; r < 4; r++)
    {
      if (r == skipR) continue;
      int cc = 0;
      for (int c = 0; c < 4; c++)
      {
        if (c == skipC) continue;
        s[rr][cc++] = a[r][c];
      }
      rr++;
    }
    const float m0 = s[1][1] * s[2][2] - s[1][2] * s[2][1];
    const float m1 = s[1][0] * s[2][2] - s[1][2] * s[2][0];
    const float m2 = s[1][0] * s[2][1] - s[1][1] * s[2][0];
    return s[0][0] * m0 - s[0][1] * m1 + s[0][2] * m2;
  };
  float cof[4][4];
  for (int r = 0; r < 4; r++)
    for (int c = 0; c < 4; c++) cof[r][c] = (((r + c) & 1) ? -1.0f : 1.0f) * minor3(r, c);
  const float det = a[0][0] * cof[0][0] + a[0][1] * cof[0][1] + a[0][2] * cof[0][2] + a[0][3] * cof[0][3];
  const float invDet = 1.0f / det;
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 4; c++) inv12[r * 4 + c] = cof[c][r] * invDet;
}

bool is_identity(const float* m)
{
  for (int c = 0; c < 4; c++)
    for (int r = 0; r < 4; r++)
    {
      const float want = (r == c) ? 1.0f : 0.0f;
      uint32_t a, b;
      std::memcpy(&a, &m[c * 4 + r], 4);
      std::memcpy(&b, &want, 4);
      if (a != b) return false;
    }
  return true;
}

int build_geometry(hrt_scene* s, Geom& g, const float* vpos, uint64_t nVert, const uint32_t* idx, uint64_t nIdx,
                   uint64_t stride, int layout, int triTest)
{
  hrt_context* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  const uint32_t N = (uint32_t)(nIdx / 3);
  g.nTris = N;
  g.triTest = triTest;
  g.nVerts = (uint32_t)nVert;
  uint64_t* bytes = &g.bytes;
  HRT_CUDA(ctx, dalloc(&g.verts, nVert, bytes, st));
  HRT_CUDA(ctx, dalloc(&g.params, 1, bytes, st));
  HRT_CUDA(ctx, cudaMemsetAsync(g.params, 0, sizeof(BuildParams), st));
  if (nVert)
  {
    if (stride == 16)
      HRT_CUDA(ctx, cudaMemcpyAsync(g.verts, vpos, 16 * nVert, cudaMemcpyDefault, st));
    uint8_t* raw = nullptr;
    if (stride != 16)
    {
      HRT_CUDA(ctx, cudaMallocAsync((void**)&raw, stride * nVert, st));
      HRT_CUDA(ctx, cudaMemcpyAsync(raw, vpos, stride * nVert, cudaMemcpyDefault, st));
    }
    const uint8_t* src = raw ? raw : reinterpret_cast<const uint8_t*>(g.verts);
    uint64_t blocks = (nVert + 255) / 256;
    if (blocks > 65535) blocks = 65535;
    k_pack_verts<<<(uint32_t)blocks, 256, 0, st>>>(src, nVert, stride, g.verts);
    HRT_CUDA(ctx, cudaGetLastError());
    if (raw) HRT_CUDA(ctx, cudaFreeAsync(raw, st));
  }
  if (N == 0)
  {
    HRT_CUDA(ctx, cudaStreamSynchronize(st));
    for (int c = 0; c < 4; c++)
    {
      g.box[c] = INFINITY;
      g.box[4 + c] = -INFINITY;
    }
    return HRT_OK;
  }

  uint32_t* dIdx = nullptr;
  uint32_t *keysAlt = nullptr, *valsAlt = nullptr, *parent = nullptr, *visit = nullptr;
  void* scratch = nullptr;
  HRT_CUDA(ctx, cudaMallocAsync((void**)&dIdx, sizeof(uint32_t) * nIdx, st));
  HRT_CUDA(ctx, cudaMemcpyAsync(dIdx, idx, sizeof(uint32_t) * nIdx, cudaMemcpyDefault, st));
  HRT_CUDA(ctx, dalloc(&g.keys, N, bytes, st));
  HRT_CUDA(ctx, dalloc(&g.vals, N, bytes, st));
  HRT_CUDA(ctx, dalloc(&g.keysUnsorted, N, bytes, st));
  HRT_CUDA(ctx, dalloc(&g.compressed, N, bytes, st));
  HRT_CUDA(ctx, dalloc(&g.runStarts, N, bytes, st));
  HRT_CUDA(ctx, dalloc(&g.lr, 2 * (size_t)N - 1, bytes, st));
  HRT_CUDA(ctx, dalloc(&g.lrCount, 2 * (size_t)N - 1, bytes, st));
  // binary pair records only for the binary layout (the 4-wide layouts
  // traverse their own nodes)
  if (layout == HRT_LAYOUT_BVH2) HRT_CUDA(ctx, dalloc(&g.recs, N > 1 ? N - 1 : 1, bytes, st));
  HRT_CUDA(ctx, dalloc(&g.tris, N, bytes, st));
  HRT_CUDA(ctx, dalloc(&g.sortedIdx, 3 * (size_t)N, bytes, st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&keysAlt, sizeof(uint32_t) * N, st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&valsAlt, sizeof(uint32_t) * N, st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&parent, sizeof(uint32_t) * (2 * (size_t)N - 1), st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&visit, sizeof(uint32_t) * 2 * (size_t)N, st));
  HRT_CUDA(ctx, cudaMallocAsync(&scratch, build_scratch_bytes(N), st));

  BuildBuffers b;
  b.verts = g.verts;
  b.idx = dIdx;
  b.nVerts = g.nVerts;
  b.nTris = N;
  b.keys = g.keys;
  b.vals = g.vals;
  b.keysAlt = keysAlt;
  b.valsAlt = valsAlt;
  b.keysUnsorted = g.keysUnsorted;
  b.compressed = g.compressed;
  b.runStarts = g.runStarts;
  b.lr = g.lr;
  b.lrCount = g.lrCount;
  b.parent = parent;
  b.visit = visit;
  b.recs = g.recs;
  b.tris = g.tris;
  b.sortedIdx = g.sortedIdx;
  b.params = g.params;
  b.scratch = scratch;
  b.vertexRecords = triTest == HRT_TRI_WATERTIGHT;
  b.mortonCubic = s->mortonFrame == HRT_MORTON_CUBIC && &g != &s->tlas;
  g.mortonFrame = b.mortonCubic ? HRT_MORTON_CUBIC : HRT_MORTON_PER_AXIS;

  cudaEvent_t e0, e1;
  HRT_CUDA(ctx, cudaEventCreate(&e0));
  HRT_CUDA(ctx, cudaEventCreate(&e1));
  HRT_CUDA(ctx, cudaEventRecord(e0, st));
  cudaError_t be = build_lbvh(b, ctx->numSMs, st);
  if (be != cudaSuccess) return cuda_fail(ctx, be, "build_lbvh");
  if (layout != HRT_LAYOUT_BVH2)
  {
    // collapse into 4-wide nodes: plan (count), allocate, emit
    void* scratch4 = nullptr;
    uint32_t count4 = 0;
    HRT_CUDA(ctx, cudaMallocAsync(&scratch4, bvh4_scratch_bytes(N), st));
    Bvh4Buffers b4;
    b4.nTris = N;
    b4.params = g.params;
    b4.lr = g.lr;
    b4.runStarts = g.runStarts;
    b4.parent = parent;
    b4.tris = g.tris;
    b4.scratch = scratch4;
    b4.mergeMode = s->bvh4Merge;
    b4.lrCount = g.lrCount;
    b4.collapse = s->bvh4Collapse;
    b4.hostNodeCount = &count4;
    g.bvh4Merge = s->bvh4Merge;
    g.bvh4Collapse = s->bvh4Collapse;
    HRT_CUDA(ctx, bvh4_plan(b4, ctx->numSMs, st));
    HRT_CUDA(ctx, cudaStreamSynchronize(st));
    if (count4 == 0) count4 = 1;  // a single leaf still gets a root node
    const size_t nodeBytes = (layout == HRT_LAYOUT_BVH4_F32) ? sizeof(Node4F32) : sizeof(Node4F16);
    HRT_CUDA(ctx, cudaMallocAsync(&g.nodes4, nodeBytes * count4, st));
    g.bytes += nodeBytes * count4;
    g.nNodes4 = count4;
    HRT_CUDA(ctx, bvh4_emit(b4, layout - 1, g.nodes4, count4, ctx->numSMs, st));
    HRT_CUDA(ctx, cudaFreeAsync(scratch4, st));
  }
  HRT_CUDA(ctx, cudaEventRecord(e1, st));
  HRT_CUDA(ctx, cudaMemcpyAsync(&g.host, g.params, sizeof(BuildParams), cudaMemcpyDeviceToHost, st));
  HRT_CUDA(ctx, cudaFreeAsync(dIdx, st));
  HRT_CUDA(ctx, cudaFreeAsync(keysAlt, st));
  HRT_CUDA(ctx, cudaFreeAsync(valsAlt, st));
  HRT_CUDA(ctx, cudaFreeAsync(parent, st));
  HRT_CUDA(ctx, cudaFreeAsync(visit, st));
  HRT_CUDA(ctx, cudaFreeAsync(scratch, st));
  HRT_CUDA(ctx, cudaStreamSynchronize(st));
  cudaEventElapsedTime(&g.buildMs, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  g.nLeaves = g.host.nLeaves;
  for (int c = 0; c < 4; c++)
  {
    g.box[c] = g.host.bmin[c];
    g.box[4 + c] = g.host.bmax[c];
  }
  const uint32_t err = g.host.error;
  if (err & kErrIndexRange) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "triangle index >= vertex count");
  if (err & kErrLeafCount)
    return fail(ctx, HRT_ERR_CAPACITY, "more than 127 triangles share one Morton code (leaf count field overflows)");
  if (err & kErrWaitTimeout) return fail(ctx, HRT_ERR_TIMEOUT, "device look-back wait timed out during the build");
  if (err & kErrLayout) return fail(ctx, HRT_ERR_DEVICE_CHECK, "inconsistent tree or node encoding");
  if (g.nLeaves == 0 || g.nLeaves > N) return fail(ctx, HRT_ERR_DEVICE_CHECK, "leaf count out of range");
  return HRT_OK;
}

// Device allocation owned by a batch: recorded in `owned` (freed together).
template <typename T> cudaError_t balloc(T** p, size_t count, std::vector<void*>& owned)
{
  const cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
  if (e == cudaSuccess) owned.push_back(*p);
  return e;
}

inline size_t align_up(size_t b, size_t a) { return (b + a - 1) / a * a; }

// Builds G geometries with one segmented LBVH build (build_batch.cu) and, for
// a 4-wide layout, collapses each.  On success appends G geometries whose
// arrays point into allocations recorded in `owned`.
int build_batch(hrt_scene* s, uint32_t G, const float* vpos, const uint64_t* vOff, const uint32_t* idx,
                const uint64_t* iOff, uint64_t stride, std::vector<Geom>& out, std::vector<void*>& owned)
{
  hrt_context* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  const uint64_t V = vOff[G], N = iOff[G] / 3;
  std::vector<uint32_t> hv(G + 1), ht(G + 1);
  for (uint32_t i = 0; i <= G; i++)
  {
    hv[i] = (uint32_t)vOff[i];
    ht[i] = (uint32_t)(iOff[i] / 3);
  }
  // inputs
  float4* verts = nullptr;
  uint32_t *dVOff = nullptr, *dTOff = nullptr, *dIdx = nullptr;
  HRT_CUDA(ctx, balloc(&verts, V, owned));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&dVOff, sizeof(uint32_t) * (G + 1), st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&dTOff, sizeof(uint32_t) * (G + 1), st));
  HRT_CUDA(ctx, cudaMemcpyAsync(dVOff, hv.data(), sizeof(uint32_t) * (G + 1), cudaMemcpyHostToDevice, st));
  HRT_CUDA(ctx, cudaMemcpyAsync(dTOff, ht.data(), sizeof(uint32_t) * (G + 1), cudaMemcpyHostToDevice, st));
  if (V)
  {
    uint8_t* raw = nullptr;
    if (stride == 16)
      HRT_CUDA(ctx, cudaMemcpyAsync(verts, vpos, 16 * V, cudaMemcpyHostToDevice, st));
    else
    {
      HRT_CUDA(ctx, cudaMallocAsync((void**)&raw, stride * V, st));
      HRT_CUDA(ctx, cudaMemcpyAsync(raw, vpos, stride * V, cudaMemcpyHostToDevice, st));
    }
    const uint8_t* src = raw ? raw : reinterpret_cast<const uint8_t*>(verts);
    uint64_t blocks = (V + 255) / 256;
    if (blocks > 65535) blocks = 65535;
    k_pack_verts<<<(uint32_t)blocks, 256, 0, st>>>(src, V, stride, verts);
    HRT_CUDA(ctx, cudaGetLastError());
    if (raw) HRT_CUDA(ctx, cudaFreeAsync(raw, st));
  }
  BatchBuffers b{};
  b.verts = verts;
  b.vertOffsets = dVOff;
  b.triOffsets = dTOff;
  b.G = G;
  b.nTris = (uint32_t)N;
  b.vertexRecords = s->triTest == HRT_TRI_WATERTIGHT;
  b.mortonCubic = s->mortonFrame == HRT_MORTON_CUBIC;
  // scene-box chunks of each geometry's vertices
  std::vector<uint32_t> hChunk(G + 1, 0);
  for (uint32_t i = 0; i < G; i++) hChunk[i + 1] = hChunk[i] + (hv[i + 1] - hv[i] + kBatchBoxChunk - 1) / kBatchBoxChunk;
  uint32_t* dChunk = nullptr;
  float4* boxPartial = nullptr;
  HRT_CUDA(ctx, cudaMallocAsync((void**)&dChunk, sizeof(uint32_t) * (G + 1), st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&boxPartial, 2 * sizeof(float4) * (hChunk[G] ? hChunk[G] : 1), st));
  HRT_CUDA(ctx, cudaMemcpyAsync(dChunk, hChunk.data(), sizeof(uint32_t) * (G + 1), cudaMemcpyHostToDevice, st));
  b.boxChunkOffsets = dChunk;
  b.nBoxChunks = hChunk[G];
  b.boxPartial = boxPartial;
  uint32_t *keysAlt = nullptr, *valsAlt = nullptr, *parent = nullptr, *visit = nullptr;
  void* scratch = nullptr;
  HRT_CUDA(ctx, balloc(&b.keys, N, owned));
  HRT_CUDA(ctx, balloc(&b.vals, N, owned));
  HRT_CUDA(ctx, balloc(&b.keysUnsorted, N, owned));
  HRT_CUDA(ctx, balloc(&b.compressed, N, owned));
  HRT_CUDA(ctx, balloc(&b.runStarts, N, owned));
  HRT_CUDA(ctx, balloc(&b.lr, 2 * N, owned));
  HRT_CUDA(ctx, balloc(&b.lrCount, 2 * N, owned));
  if (s->layout == HRT_LAYOUT_BVH2) HRT_CUDA(ctx, balloc(&b.recs, N, owned));
  HRT_CUDA(ctx, balloc(&b.tris, N, owned));
  HRT_CUDA(ctx, balloc(&b.sortedIdx, 3 * N, owned));
  HRT_CUDA(ctx, balloc(&b.params, G, owned));
  // offsets (4 x (G+1)), counts (4) and the error word in one array
  uint32_t* offs = nullptr;
  HRT_CUDA(ctx, balloc(&offs, 4 * ((size_t)G + 1) + 8, owned));
  b.leafOffsets = offs;
  b.intOffsets = offs + (G + 1);
  b.nodeOffsets = offs + 2 * (G + 1);
  b.recOffsets = offs + 3 * (G + 1);
  b.counts = offs + 4 * (G + 1);
  b.errorWord = b.counts + 4;
  HRT_CUDA(ctx, cudaMemsetAsync(offs, 0, sizeof(uint32_t) * (4 * ((size_t)G + 1) + 8), st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&dIdx, sizeof(uint32_t) * 3 * (N ? N : 1), st));
  if (N) HRT_CUDA(ctx, cudaMemcpyAsync(dIdx, idx, sizeof(uint32_t) * 3 * N, cudaMemcpyHostToDevice, st));
  b.idx = dIdx;
  HRT_CUDA(ctx, cudaMallocAsync((void**)&keysAlt, sizeof(uint32_t) * (N ? N : 1), st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&valsAlt, sizeof(uint32_t) * (N ? N : 1), st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&parent, sizeof(uint32_t) * 2 * (N ? N : 1), st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&visit, sizeof(uint32_t) * 2 * (N ? N : 1), st));
  HRT_CUDA(ctx, cudaMallocAsync(&scratch, build_batch_scratch_bytes((uint32_t)N, G), st));
  b.keysAlt = keysAlt;
  b.valsAlt = valsAlt;
  b.parent = parent;
  b.visit = visit;
  b.scratch = scratch;
  if (N == 0) HRT_CUDA(ctx, cudaMemsetAsync(b.params, 0, sizeof(BuildParams) * G, st));

  cudaEvent_t e0, e1;
  HRT_CUDA(ctx, cudaEventCreate(&e0));
  HRT_CUDA(ctx, cudaEventCreate(&e1));
  HRT_CUDA(ctx, cudaEventRecord(e0, st));
  cudaError_t be = build_lbvh_batch(b, ctx->numSMs, st);
  if (be != cudaSuccess) return cuda_fail(ctx, be, "build_lbvh_batch");
  std::vector<BuildParams> hp(G);
  std::vector<uint32_t> ho(4 * ((size_t)G + 1) + 8);
  HRT_CUDA(ctx, cudaMemcpyAsync(ho.data(), offs, sizeof(uint32_t) * ho.size(), cudaMemcpyDeviceToHost, st));
  HRT_CUDA(ctx, cudaMemcpyAsync(hp.data(), b.params, sizeof(BuildParams) * G, cudaMemcpyDeviceToHost, st));
  HRT_CUDA(ctx, cudaStreamSynchronize(st));
  const uint32_t* hLeaf = ho.data();
  const uint32_t* hNode = ho.data() + 2 * (G + 1);
  const uint32_t* hRec = ho.data() + 3 * (G + 1);
  uint32_t err = ho[4 * ((size_t)G + 1) + 4];

  // 4-wide collapse of every geometry at once: plan (one launch per stage over
  // the whole batch), one synchronisation for the node counts, then emit into
  // one node array
  std::vector<uint32_t> count4(G, 0);
  std::vector<size_t> node4Off(G, 0);
  void* nodes4 = nullptr;
  size_t nodeBytes = 0;
  void* scratch4 = nullptr;
  if (s->layout != HRT_LAYOUT_BVH2 && N > 0 && err == 0)
  {
    nodeBytes = (s->layout == HRT_LAYOUT_BVH4_F32) ? sizeof(Node4F32) : sizeof(Node4F16);
    const uint32_t* hInt = ho.data() + (G + 1);
    const uint32_t nInt = hInt[G];
    Bvh4Batch q;
    q.G = G;
    q.lr = b.lr;
    q.runStarts = b.runStarts;
    q.parent = parent;
    q.tris = b.tris;
    q.leafOffsets = b.leafOffsets;
    q.intOffsets = b.intOffsets;
    q.nodeOffsets = b.nodeOffsets;
    q.triOffsets = b.triOffsets;
    q.lrCount = b.lrCount;
    q.mergeMode = s->bvh4Merge;
    q.collapse = s->bvh4Collapse;
    HRT_CUDA(ctx, cudaMallocAsync(&scratch4, bvh4_batch_scratch_bytes(nInt, G), st));
    uint32_t* hostCounts = nullptr;
    HRT_CUDA(ctx, cudaMallocHost((void**)&hostCounts, sizeof(uint32_t) * (2 * (size_t)G + 1)));
    cudaError_t pe = bvh4_plan_batch(q, nInt, scratch4, hostCounts, hostCounts + G, b.errorWord, ctx->numSMs, st);
    if (pe == cudaSuccess) pe = cudaStreamSynchronize(st);
    if (pe != cudaSuccess)
    {
      cudaFreeHost(hostCounts);
      return cuda_fail(ctx, pe, "bvh4_plan_batch");
    }
    for (uint32_t i = 0; i < G; i++)
    {
      count4[i] = hostCounts[i];
      node4Off[i] = hostCounts[G + i];
    }
    const size_t total = hostCounts[2 * (size_t)G];
    cudaFreeHost(hostCounts);
    HRT_CUDA(ctx, balloc((char**)&nodes4, nodeBytes * (total ? total : 1), owned));
    HRT_CUDA(ctx, bvh4_emit_batch(q, nInt, scratch4, s->layout - 1, nodes4, b.errorWord, ctx->numSMs, st));
  }
  HRT_CUDA(ctx, cudaEventRecord(e1, st));
  uint32_t collapseErr = 0;
  if (nodes4)
  {
    HRT_CUDA(ctx, cudaMemcpyAsync(hp.data(), b.params, sizeof(BuildParams) * G, cudaMemcpyDeviceToHost, st));
    HRT_CUDA(ctx, cudaMemcpyAsync(&collapseErr, b.errorWord, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  }
  HRT_CUDA(ctx, cudaFreeAsync(dIdx, st));
  HRT_CUDA(ctx, cudaFreeAsync(keysAlt, st));
  HRT_CUDA(ctx, cudaFreeAsync(valsAlt, st));
  HRT_CUDA(ctx, cudaFreeAsync(parent, st));
  HRT_CUDA(ctx, cudaFreeAsync(visit, st));
  HRT_CUDA(ctx, cudaFreeAsync(scratch, st));
  HRT_CUDA(ctx, cudaFreeAsync(dVOff, st));
  HRT_CUDA(ctx, cudaFreeAsync(dTOff, st));
  HRT_CUDA(ctx, cudaFreeAsync(dChunk, st));
  HRT_CUDA(ctx, cudaFreeAsync(boxPartial, st));
  if (scratch4) HRT_CUDA(ctx, cudaFreeAsync(scratch4, st));
  HRT_CUDA(ctx, cudaStreamSynchronize(st));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  err |= collapseErr;
  for (uint32_t i = 0; i < G; i++) err |= hp[i].error;
  if (err & kErrIndexRange) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "triangle index >= vertex count of its geometry");
  if (err & kErrLeafCount)
    return fail(ctx, HRT_ERR_CAPACITY, "more than 127 triangles share one Morton code (leaf count field overflows)");
  if (err & kErrWaitTimeout) return fail(ctx, HRT_ERR_TIMEOUT, "device look-back wait timed out during the build");
  if (err & kErrLayout) return fail(ctx, HRT_ERR_DEVICE_CHECK, "inconsistent tree or node encoding");

  out.resize(G);
  for (uint32_t i = 0; i < G; i++)
  {
    Geom& g = out[i];
    const uint32_t Ni = ht[i + 1] - ht[i];
    const uint32_t Li = hLeaf[i + 1] - hLeaf[i];
    g.shared = true;
    g.bvh4Merge = s->bvh4Merge;
    g.bvh4Collapse = s->bvh4Collapse;
    g.triTest = s->triTest;
    g.mortonFrame = s->mortonFrame;
    g.nTris = Ni;
    g.nVerts = hv[i + 1] - hv[i];
    g.nLeaves = Li;
    g.verts = verts + hv[i];
    g.keys = b.keys + ht[i];
    g.vals = b.vals + ht[i];
    g.keysUnsorted = b.keysUnsorted + ht[i];
    g.compressed = b.compressed + hLeaf[i];
    g.runStarts = b.runStarts + hLeaf[i];
    g.lr = b.lr + hNode[i];
    g.lrCount = b.lrCount + hNode[i];
    g.recs = b.recs ? b.recs + hRec[i] : nullptr;
    g.tris = b.tris + ht[i];
    g.sortedIdx = b.sortedIdx + 3 * (size_t)ht[i];
    g.params = b.params + i;
    g.host = hp[i];
    g.buildMs = ms;  // the whole batch's build time
    if (nodes4 && count4[i])
    {
      g.nodes4 = (char*)nodes4 + nodeBytes * node4Off[i];
      g.nNodes4 = count4[i];
    }
    const uint64_t recsI = Li > 1 ? Li - 1 : (Li ? 1 : 0);
    g.bytes = 16ull * g.nVerts + (uint64_t)Ni * (4 * 5 + sizeof(TriRec) + 12) + (Li ? (2ull * Li - 1) * 36 : 0) +
              recsI * sizeof(PairRec) + (uint64_t)g.nNodes4 * nodeBytes + sizeof(BuildParams);
    if (Ni == 0)
      for (int c = 0; c < 4; c++)
      {
        g.box[c] = INFINITY;
        g.box[4 + c] = -INFINITY;
      }
    else
    {
      if (Li == 0 || Li > Ni) return fail(ctx, HRT_ERR_DEVICE_CHECK, "leaf count out of range");
      for (int c = 0; c < 4; c++)
      {
        g.box[c] = hp[i].bmin[c];
        g.box[4 + c] = hp[i].bmax[c];
      }
    }
  }
  return HRT_OK;
}

void make_instance_desc(const Geom& g, uint32_t geomId, uint32_t instId, const float* inv12, InstanceDesc& d)
{
  static const float id12[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  d.recs = g.recs;
  d.nodes4 = g.nodes4;
  d.tris = g.tris;
  d.geomId = geomId;
  d.instId = instId;
  d.identity = inv12 ? 0u : 1u;
  d.valid = g.nTris > 0 ? 1u : 0u;
  std::memcpy(d.inv, inv12 ? inv12 : id12, sizeof(d.inv));
}

// World-space box of an instance: the geometry's box corners under the
// instance matrix, evaluated in double, rounded outward to float and widened
// by a relative margin that covers the rounding of the rays' transform into
// the instance.
void instance_world_box(const Geom& g, const float* m, float* mn, float* mx)
{
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int corner = 0; corner < 8; corner++)
  {
    const double p[3] = {g.box[(corner & 1) ? 4 : 0], g.box[(corner & 2) ? 5 : 1], g.box[(corner & 4) ? 6 : 2]};
    for (int r = 0; r < 3; r++)
    {
      const double v = (double)m[r] * p[0] + (double)m[4 + r] * p[1] + (double)m[8 + r] * p[2] + (double)m[12 + r];
      lo[r] = std::min(lo[r], v);
      hi[r] = std::max(hi[r], v);
    }
  }
  for (int r = 0; r < 3; r++)
  {
    const double margin = 1e-5 * (hi[r] - lo[r]) + 1e-6 * std::max(std::fabs(lo[r]), std::fabs(hi[r])) + 1e-30;
    mn[r] = std::nextafter((float)(lo[r] - margin), -INFINITY);
    mx[r] = std::nextafter((float)(hi[r] + margin), INFINITY);
  }
}

// Instance tree of the scene's instances with triangles: one pseudo-triangle
// per instance (min corner, max corner, max corner) whose box is the
// instance's world box, built by the geometry LBVH build in the binary
// layout.  Triangle record e1.w (the pseudo-triangle's index) is rewritten to
// the instance id.  Leaves may hold more than 127 instances (coincident
// instances share a Morton code): the traversal ends a leaf at its flagged
// record, so only the exported LR leaf count would overflow.
int build_tlas(hrt_scene* s)
{
  std::vector<uint32_t> ids;
  for (size_t i = 0; i < s->insts.size(); i++)
    if (s->geoms[s->insts[i].geomId].nTris > 0) ids.push_back((uint32_t)i);
  const size_t n = ids.size();
  if (n == 0) return HRT_OK;  // nothing to hit
  std::vector<float> v(12 * n);
  std::vector<uint32_t> idx(3 * n);
  for (size_t j = 0; j < n; j++)
  {
    const Instance& in = s->insts[ids[j]];
    float mn[3], mx[3];
    instance_world_box(s->geoms[in.geomId], in.m, mn, mx);
    for (int r = 0; r < 3; r++)
    {
      v[12 * j + r] = mn[r];
      v[12 * j + 4 + r] = mx[r];
      v[12 * j + 8 + r] = mx[r];
    }
    v[12 * j + 3] = v[12 * j + 7] = v[12 * j + 11] = 1.0f;
    for (int c = 0; c < 3; c++) idx[3 * j + c] = (uint32_t)(3 * j + c);
  }
  int st = build_geometry(s, s->tlas, v.data(), 3 * n, idx.data(), 3 * n, 16, HRT_LAYOUT_BVH2);
  if (st == HRT_ERR_CAPACITY && (s->tlas.host.error & ~kErrLeafCount) == 0 && s->tlas.nLeaves > 0 &&
      s->tlas.nLeaves <= n)
    st = HRT_OK;
  if (st != HRT_OK) return st;
  std::vector<TriRec> tr(n);
  HRT_CUDA(s->ctx, cudaMemcpy(tr.data(), s->tlas.tris, sizeof(TriRec) * n, cudaMemcpyDeviceToHost));
  for (TriRec& r : tr)
  {
    uint32_t k;
    std::memcpy(&k, &r.e1.w, 4);
    if (k >= n) return fail(s->ctx, HRT_ERR_DEVICE_CHECK, "instance tree record out of range");
    std::memcpy(&r.e1.w, &ids[k], 4);
  }
  HRT_CUDA(s->ctx, cudaMemcpy(s->tlas.tris, tr.data(), sizeof(TriRec) * n, cudaMemcpyHostToDevice));
  return HRT_OK;
}

// Copies nVert host vertices of `stride` bytes (xyz first) to float4 (w = 1) on the device.
int upload_verts(hrt_context* ctx, cudaStream_t st, float4* dst, const float* vpos, uint64_t nVert, uint64_t stride)
{
  if (nVert == 0) return HRT_OK;
  if (stride == 16) HRT_CUDA(ctx, cudaMemcpyAsync(dst, vpos, 16 * nVert, cudaMemcpyHostToDevice, st));
  uint8_t* raw = nullptr;
  if (stride != 16)
  {
    HRT_CUDA(ctx, cudaMallocAsync((void**)&raw, stride * nVert, st));
    HRT_CUDA(ctx, cudaMemcpyAsync(raw, vpos, stride * nVert, cudaMemcpyHostToDevice, st));
  }
  uint64_t blocks = (nVert + 255) / 256;
  if (blocks > 65535) blocks = 65535;
  k_pack_verts<<<(uint32_t)blocks, 256, 0, st>>>(raw ? raw : reinterpret_cast<const uint8_t*>(dst), nVert, stride, dst);
  HRT_CUDA(ctx, cudaGetLastError());
  if (raw) HRT_CUDA(ctx, cudaFreeAsync(raw, st));
  return HRT_OK;
}

// Refit of geometry g to new vertex positions (same vertex and index counts,
// same index buffer): the build's tree topology and sorted order are kept,
// every box, triangle record and traversal record is recomputed, and a 4-wide
// layout is collapsed again into the same node array.
int refit_geometry(hrt_scene* s, Geom& g, const float* vpos, const uint32_t* idx, uint64_t stride)
{
  hrt_context* ctx = s->ctx;
  cudaStream_t st = ctx->stream;
  const uint32_t N = g.nTris;
  int rc = upload_verts(ctx, st, g.verts, vpos, g.nVerts, stride);
  if (rc != HRT_OK) return rc;
  if (N == 0)
  {
    HRT_CUDA(ctx, cudaStreamSynchronize(st));
    return HRT_OK;
  }
  uint32_t *dIdx = nullptr, *parent = nullptr, *visit = nullptr;
  BuildParams* box = nullptr;
  void* scratch = nullptr;
  HRT_CUDA(ctx, cudaMallocAsync((void**)&dIdx, sizeof(uint32_t) * 3 * (size_t)N, st));
  HRT_CUDA(ctx, cudaMemcpyAsync(dIdx, idx, sizeof(uint32_t) * 3 * (size_t)N, cudaMemcpyHostToDevice, st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&parent, sizeof(uint32_t) * (2 * (size_t)N - 1), st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&visit, sizeof(uint32_t) * 2 * (size_t)N, st));
  HRT_CUDA(ctx, cudaMallocAsync((void**)&box, sizeof(BuildParams), st));
  HRT_CUDA(ctx, cudaMallocAsync(&scratch, refit_scratch_bytes(), st));
  HRT_CUDA(ctx, cudaMemsetAsync(&g.params->error, 0, sizeof(uint32_t), st));
  BuildBuffers b{};
  b.verts = g.verts;
  b.idx = dIdx;
  b.nVerts = g.nVerts;
  b.nTris = N;
  b.vals = g.vals;
  b.compressed = g.compressed;
  b.runStarts = g.runStarts;
  b.lr = g.lr;
  b.lrCount = g.lrCount;
  b.parent = parent;
  b.visit = visit;
  b.recs = g.recs;
  b.tris = g.tris;
  b.sortedIdx = g.sortedIdx;
  b.params = g.params;
  b.scratch = scratch;
  b.vertexRecords = g.triTest == HRT_TRI_WATERTIGHT;
  b.mortonCubic = g.mortonFrame == HRT_MORTON_CUBIC;  // only the vertex box is recomputed
  cudaEvent_t e0, e1;
  HRT_CUDA(ctx, cudaEventCreate(&e0));
  HRT_CUDA(ctx, cudaEventCreate(&e1));
  HRT_CUDA(ctx, cudaEventRecord(e0, st));
  cudaError_t e = refit_lbvh(b, box, ctx->numSMs, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "refit_lbvh");
  if (s->layout != HRT_LAYOUT_BVH2)
  {
    void* scratch4 = nullptr;
    uint32_t count4 = 0;
    HRT_CUDA(ctx, cudaMallocAsync(&scratch4, bvh4_scratch_bytes(N), st));
    Bvh4Buffers b4;
    b4.nTris = N;
    b4.params = g.params;
    b4.lr = g.lr;
    b4.runStarts = g.runStarts;
    b4.parent = parent;
    b4.tris = g.tris;
    b4.scratch = scratch4;
    b4.mergeMode = g.bvh4Merge;
    b4.lrCount = g.lrCount;
    b4.collapse = g.bvh4Collapse;
    b4.hostNodeCount = &count4;
    HRT_CUDA(ctx, bvh4_plan(b4, ctx->numSMs, st));
    HRT_CUDA(ctx, cudaStreamSynchronize(st));
    if (count4 == 0) count4 = 1;
    if (count4 != g.nNodes4) return fail(ctx, HRT_ERR_DEVICE_CHECK, "refit changed the 4-wide node count");
    HRT_CUDA(ctx, bvh4_emit(b4, s->layout - 1, g.nodes4, count4, ctx->numSMs, st));
    HRT_CUDA(ctx, cudaFreeAsync(scratch4, st));
  }
  HRT_CUDA(ctx, cudaEventRecord(e1, st));
  BuildParams hb{}, hp{};
  HRT_CUDA(ctx, cudaMemcpyAsync(&hb, box, sizeof(BuildParams), cudaMemcpyDeviceToHost, st));
  HRT_CUDA(ctx, cudaMemcpyAsync(&hp, g.params, sizeof(BuildParams), cudaMemcpyDeviceToHost, st));
  HRT_CUDA(ctx, cudaFreeAsync(dIdx, st));
  HRT_CUDA(ctx, cudaFreeAsync(parent, st));
  HRT_CUDA(ctx, cudaFreeAsync(visit, st));
  HRT_CUDA(ctx, cudaFreeAsync(box, st));
  HRT_CUDA(ctx, cudaFreeAsync(scratch, st));
  HRT_CUDA(ctx, cudaStreamSynchronize(st));
  cudaEventElapsedTime(&g.buildMs, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (hp.error & kErrIndexRange) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "triangle index >= vertex count");
  if (hp.error & (kErrLayout | kErrLeafCount)) return fail(ctx, HRT_ERR_DEVICE_CHECK, "inconsistent tree after refit");
  for (int c = 0; c < 4; c++)
  {
    g.box[c] = hb.bmin[c];
    g.box[4 + c] = hb.bmax[c];
  }
  return HRT_OK;
}

bool lbvh_builder_name(const char* name)
{
  if (!name || !*name) return true;
  const std::string s(name);
  return s.find("lbvh") != std::string::npos;  // "cbvh_lbvh", "lbvh", "cbvh_lbvh_gpu" (core/builders/cbvh.cpp:45-55)
}

// Whether the current device reaches pageable host memory through the host's
// own page tables (address translation over NVLink-C2C on Grace-based
// systems), so that a kernel may read and write such memory where it is;
// cached per device.
bool pageable_access()
{
  static std::atomic<int> known[64];  // 0 not asked yet, 1 no, 2 yes
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
  {
    cudaGetLastError();
    return false;
  }
  int k = known[dev].load(std::memory_order_relaxed);
  if (k == 0)
  {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess)
    {
      cudaGetLastError();
      v = 0;
    }
    k = v ? 2 : 1;
    known[dev].store(k, std::memory_order_relaxed);
  }
  return k == 2;
}

void* mapped_host(const void* p, bool pageable)
{
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
  {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost) return a.devicePointer;
  if (pageable && a.type == cudaMemoryTypeUnregistered && pageable_access()) return const_cast<void*>(p);
  return nullptr;
}

int ensure_stage(hrt_scene* s, uint64_t n)
{
  if (n <= s->stageCap) return HRT_OK;
  if (s->stageRays) cudaFree(s->stageRays);
  if (s->stageOut) cudaFree(s->stageOut);
  s->stageRays = s->stageOut = nullptr;
  s->stageCap = 0;
  HRT_CUDA(s->ctx, cudaMalloc(&s->stageRays, 32 * n));
  HRT_CUDA(s->ctx, cudaMalloc(&s->stageOut, sizeof(hrt_hit) * n));
  s->stageCap = n;
  return HRT_OK;
}

// Segments of a segmented query (all null/0 for a plain query) and, when not
// null, the work counter the launch uses instead of a slot of the scene's ring.
struct QuerySegments
{
  const uint32_t*    rayOffsets = nullptr;
  const uint32_t*    segInst = nullptr;
  uint32_t           nSeg = 0;
  unsigned int*      counter = nullptr;
  const TraceConfig* config = nullptr;  // launch shape for this launch instead of the scene's
};

int launch_query(hrt_scene* s, int kind, const float* rays, uint64_t n, void* out, int counting, cudaStream_t st,
                 const QuerySegments& q = QuerySegments())
{
  if (!s->committed) return fail(s->ctx, HRT_ERR_STATE, "query before hrt_commit_scene");
  if ((rays && !aligned_to(rays, 16)) || (kind == 0 && out && !aligned_to(out, 16)))
    return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "ray and hit arrays must be 16-byte aligned");
  if (n == 0) return HRT_OK;
  if (!rays || !out) return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "null ray or output pointer");
  if (n > 0xFFFFFFFFull) return fail(s->ctx, HRT_ERR_CAPACITY, "more than 2^32-1 rays in one query");
  if (q.rayOffsets && (!q.segInst || q.nSeg == 0))
    return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "segmented query without segments");
  TraceArgs a;
  a.rays = reinterpret_cast<const float4*>(rays);
  a.n = n;
  a.inst = s->dInst;
  a.nInst = s->nInstDev;
  a.hits = out;
  a.counters = s->dCounters;
  a.errorWord = s->dError;
  a.rayCounter = q.counter ? q.counter : s->dRayCounters + (s->counterSlot.fetch_add(1) % kCounterSlots);
  a.rayOffsets = q.rayOffsets;
  a.segInst = q.segInst;
  a.nSeg = q.nSeg;
  if (s->tlas.nTris > 0)
  {
    a.tlasRecs = s->tlas.recs;
    a.tlasTris = s->tlas.tris;
  }
  if (s->single && !q.rayOffsets) a.one = &s->singleDesc;
  a.triTest = s->triTest;
  if (a.one && s->l2PersistMB > 0)
  {
    // L2 window over the geometry's nodes: as much of the array as the
    // device's window and the persisting set-aside hold, the share of it
    // that fits the set-aside marked persisting
    int maxWin = 0, maxPersist = 0;
    cudaDeviceGetAttribute(&maxWin, cudaDevAttrMaxAccessPolicyWindowSize, s->ctx->device);
    cudaDeviceGetAttribute(&maxPersist, cudaDevAttrMaxPersistingL2CacheSize, s->ctx->device);
    const size_t setAside = std::min<size_t>((size_t)s->l2PersistMB << 20, (size_t)maxPersist);
    a.persistBase = s->layout == HRT_LAYOUT_BVH2 ? static_cast<const void*>(s->singleDesc.recs) : s->singleDesc.nodes4;
    a.persistBytes = std::min<size_t>(s->singleNodeBytes, (size_t)maxWin);
    a.persistHitRatio = a.persistBytes ? std::min(1.0f, (float)setAside / (float)a.persistBytes) : 0.0f;
    if (setAside == 0) a.persistBytes = 0;
  }
  cudaError_t e = trace(a, kind, counting, s->layout, q.config ? *q.config : s->cfg[kind], s->ctx->numSMs, st);
  if (e != cudaSuccess) return cuda_fail(s->ctx, e, "trace launch");
  return HRT_OK;
}

}  // namespace api
}  // namespace hrt

extern "C" {

const char* hrt_version(void) { return "heavyrt-gb300 0.1 (sm_103a)"; }

const char* hrt_status_string(int status)
{
  switch (status)
  {
    case HRT_OK: return "ok";
    case HRT_ERR_INVALID_ARGUMENT: return "invalid argument";
    case HRT_ERR_CUDA: return "CUDA error";
    case HRT_ERR_OUT_OF_MEMORY: return "out of device memory";
    case HRT_ERR_CAPACITY: return "format capacity exceeded";
    case HRT_ERR_STATE: return "call out of order";
    case HRT_ERR_TIMEOUT: return "device wait timed out";
    case HRT_ERR_DEVICE_CHECK: return "device-side check failed";
    case HRT_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

int hrt_context_create(int device, hrt_context** out)
{
  if (!out) return HRT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) return HRT_ERR_CUDA;
  if (device < 0 || device >= count) return HRT_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return HRT_ERR_CUDA;
  hrt_context* c = new hrt_context();
  c->device = device;
  cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, device);
  // keep up to 2 GiB of freed stream-ordered memory in the device's pool, so
  // that build scratch arrays and geometry arrays are reused instead of being
  // returned to the driver at every synchronisation
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess)
  {
    uint64_t threshold = 0;
    if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold) == cudaSuccess &&
        threshold < (2ull << 30))
    {
      threshold = 2ull << 30;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
  }
  cudaGetLastError();
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
  {
    delete c;
    return HRT_ERR_CUDA;
  }
  *out = c;
  return HRT_OK;
}

int hrt_context_destroy(hrt_context* ctx)
{
  if (!ctx) return HRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return HRT_OK;
}

const char* hrt_context_last_error(const hrt_context* ctx) { return ctx ? ctx->lastError.c_str() : "null context"; }

int hrt_scene_create(hrt_context* ctx, const char* buildName, hrt_scene** out)
{
  if (!ctx || !out) return HRT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!lbvh_builder_name(buildName))
    return fail(ctx, HRT_ERR_UNSUPPORTED, std::string("builder '") + buildName + "' is not an LBVH builder");
  cudaSetDevice(ctx->device);
  hrt_scene* s = new hrt_scene();
  s->ctx = ctx;
  // error word + the state of the first ray that ran out of its step budget
  if (cudaMalloc((void**)&s->dError, 8 * sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc((void**)&s->dCounters, 2 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc((void**)&s->dRayCounters, kCounterSlots * sizeof(unsigned int)) != cudaSuccess ||
      cudaMemset(s->dError, 0, 8 * sizeof(uint32_t)) != cudaSuccess)
  {
    if (s->dError) cudaFree(s->dError);
    if (s->dCounters) cudaFree(s->dCounters);
    if (s->dRayCounters) cudaFree(s->dRayCounters);
    delete s;
    return fail(ctx, HRT_ERR_OUT_OF_MEMORY, "scene allocation");
  }
  *out = s;
  return HRT_OK;
}

int hrt_clear_geom(hrt_scene* s)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->mu);
  cudaSetDevice(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  for (Geom& gm : s->geoms) free_geom(gm);
  free_geom(s->tlas);
  for (void* p : s->batchAllocs) cudaFree(p);
  s->batchAllocs.clear();
  s->geoms.clear();
  s->insts.clear();
  s->committed = false;
  return HRT_OK;
}

int hrt_scene_destroy(hrt_scene* s)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  hrt_clear_geom(s);
  if (s->dInst) cudaFree(s->dInst);
  if (s->dError) cudaFree(s->dError);
  if (s->dCounters) cudaFree(s->dCounters);
  if (s->dRayCounters) cudaFree(s->dRayCounters);
  if (s->stageRays) cudaFree(s->stageRays);
  if (s->stageOut) cudaFree(s->stageOut);
  for (cudaStream_t p : s->pipe)
    if (p) cudaStreamDestroy(p);
  delete s;
  return HRT_OK;
}

int hrt_add_geom_triangles3f(hrt_scene* s, const float* vpos, uint64_t nVert, const uint32_t* idx, uint64_t nIdx,
                             int quality, uint64_t vByteStride, uint32_t* geomId)
{
  (void)quality;
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = s->ctx;
  if (vByteStride == 0) vByteStride = 12;
  if (vByteStride < 12 || vByteStride % 4 != 0) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "vByteStride must be >= 12 and a multiple of 4");
  if (nIdx % 3 != 0) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "index count is not a multiple of 3");
  if ((nVert && !vpos) || (nIdx && !idx)) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "null vertex or index pointer");
  if (nIdx / 3 > HRT_MAX_TRIS_PER_GEOM) return fail(ctx, HRT_ERR_CAPACITY, "more than 2^24-1 triangles in one geometry");
  if (nVert > 0xFFFFFFFFull) return fail(ctx, HRT_ERR_CAPACITY, "more than 2^32-1 vertices in one geometry");
  std::lock_guard<std::mutex> lk(s->mu);
  cudaSetDevice(ctx->device);
  Geom g;
  const int st = build_geometry(s, g, vpos, nVert, idx, nIdx, vByteStride, s->layout, s->triTest);
  if (st != HRT_OK)
  {
    cudaStreamSynchronize(ctx->stream);
    free_geom(g);
    return st;
  }
  s->geoms.push_back(g);
  s->committed = false;
  if (geomId) *geomId = (uint32_t)(s->geoms.size() - 1);
  return HRT_OK;
}

int hrt_add_geoms_triangles3f_batched(hrt_scene* s, uint32_t count, const float* vpos, const uint64_t* vertOffsets,
                                      const uint32_t* idx, const uint64_t* idxOffsets, int quality,
                                      uint64_t vByteStride, uint32_t* firstGeomId)
{
  (void)quality;
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = s->ctx;
  if (count == 0) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "empty batch");
  if (!vertOffsets || !idxOffsets) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "null offset array");
  if (vByteStride == 0) vByteStride = 12;
  if (vByteStride < 12 || vByteStride % 4 != 0)
    return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "vByteStride must be >= 12 and a multiple of 4");
  if (vertOffsets[0] != 0 || idxOffsets[0] != 0) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "offsets must start at 0");
  for (uint32_t i = 0; i < count; i++)
  {
    if (vertOffsets[i + 1] < vertOffsets[i] || idxOffsets[i + 1] < idxOffsets[i])
      return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "offsets must be ascending");
    if ((idxOffsets[i + 1] - idxOffsets[i]) % 3 != 0)
      return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "a geometry's index count is not a multiple of 3");
    if ((idxOffsets[i + 1] - idxOffsets[i]) / 3 > HRT_MAX_TRIS_PER_GEOM)
      return fail(ctx, HRT_ERR_CAPACITY, "more than 2^24-1 triangles in one geometry");
  }
  const uint64_t V = vertOffsets[count], nIdx = idxOffsets[count];
  if ((V && !vpos) || (nIdx && !idx)) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "null vertex or index pointer");
  if (nIdx / 3 > HRT_MAX_TRIS_PER_BATCH) return fail(ctx, HRT_ERR_CAPACITY, "more than 2^30-1 triangles in one batch");
  if (V > 0xFFFFFFFFull) return fail(ctx, HRT_ERR_CAPACITY, "more than 2^32-1 vertices in one batch");
  std::lock_guard<std::mutex> lk(s->mu);
  cudaSetDevice(ctx->device);
  std::vector<Geom> built;
  std::vector<void*> owned;
  const int st = build_batch(s, count, vpos, vertOffsets, idx, idxOffsets, vByteStride, built, owned);
  if (st != HRT_OK)
  {
    cudaStreamSynchronize(ctx->stream);
    for (void* p : owned) cudaFree(p);
    return st;
  }
  const uint32_t first = (uint32_t)s->geoms.size();
  for (Geom& g : built) s->geoms.push_back(g);
  for (void* p : owned) s->batchAllocs.push_back(p);
  s->committed = false;
  if (firstGeomId) *firstGeomId = first;
  return HRT_OK;
}

int hrt_update_geom_triangles3f(hrt_scene* s, uint32_t geomId, const float* vpos, uint64_t nVert, const uint32_t* idx,
                                uint64_t nIdx, int quality, uint64_t vByteStride)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = s->ctx;
  if (vByteStride == 0) vByteStride = 12;
  if (vByteStride < 12 || vByteStride % 4 != 0)
    return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "vByteStride must be >= 12 and a multiple of 4");
  if (nIdx % 3 != 0) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "index count is not a multiple of 3");
  if ((nVert && !vpos) || (nIdx && !idx)) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "null vertex or index pointer");
  if (nIdx / 3 > HRT_MAX_TRIS_PER_GEOM) return fail(ctx, HRT_ERR_CAPACITY, "more than 2^24-1 triangles in one geometry");
  if (nVert > 0xFFFFFFFFull) return fail(ctx, HRT_ERR_CAPACITY, "more than 2^32-1 vertices in one geometry");
  std::lock_guard<std::mutex> lk(s->mu);
  if (geomId >= s->geoms.size()) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "unknown geometry id");
  cudaSetDevice(ctx->device);
  Geom& g = s->geoms[geomId];
  int st;
  if (quality == HRT_BUILD_REFIT)
  {
    if (nVert != g.nVerts || nIdx != 3 * (uint64_t)g.nTris)
      return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "a refit keeps the geometry's vertex and index counts");
    st = refit_geometry(s, g, vpos, idx, vByteStride);
  }
  else
  {
    if (g.shared)
      return fail(ctx, HRT_ERR_UNSUPPORTED, "a batch-built geometry can only be refit (BUILD_REFIT)");
    Geom ng;
    st = build_geometry(s, ng, vpos, nVert, idx, nIdx, vByteStride, s->layout, s->triTest);
    cudaStreamSynchronize(ctx->stream);
    if (st == HRT_OK)
    {
      free_geom(g);
      g = ng;
    }
    else
      free_geom(ng);
  }
  s->committed = false;  // instance descriptors and the instance tree see the new geometry at the next commit
  return st;
}

int hrt_clear_scene(hrt_scene* s)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->mu);
  cudaSetDevice(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  free_geom(s->tlas);
  s->insts.clear();
  s->committed = false;
  return HRT_OK;
}

int hrt_add_instance(hrt_scene* s, uint32_t geomId, const float m[16], uint32_t* instId)
{
  if (!s || !m) return HRT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->mu);
  if (geomId >= s->geoms.size()) return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "unknown geometry id");
  Instance in;
  in.geomId = geomId;
  std::memcpy(in.m, m, sizeof(in.m));
  in.identity = is_identity(m);
  if (in.identity)
  {
    const float id12[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    std::memcpy(in.inv, id12, sizeof(id12));
  }
  else
    inverse4x4(m, in.inv);
  s->insts.push_back(in);
  s->committed = false;
  if (instId) *instId = (uint32_t)(s->insts.size() - 1);
  return HRT_OK;
}

int hrt_update_instance(hrt_scene* s, uint32_t instId, const float m[16])
{
  if (!s || !m) return HRT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->mu);
  if (instId >= s->insts.size()) return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "unknown instance id");
  Instance& in = s->insts[instId];
  std::memcpy(in.m, m, sizeof(in.m));
  in.identity = is_identity(m);
  if (!in.identity) inverse4x4(m, in.inv);
  else
  {
    const float id12[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    std::memcpy(in.inv, id12, sizeof(id12));
  }
  s->committed = false;
  return HRT_OK;
}

int hrt_commit_scene(hrt_scene* s, int quality)
{
  (void)quality;
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->mu);
  hrt_context* ctx = s->ctx;
  cudaSetDevice(ctx->device);
  std::vector<InstanceDesc> d(s->insts.size());
  for (size_t i = 0; i < s->insts.size(); i++)
  {
    const Instance& in = s->insts[i];
    make_instance_desc(s->geoms[in.geomId], in.geomId, (uint32_t)i, in.identity ? nullptr : in.inv, d[i]);
  }
  free_geom(s->tlas);
  if (s->useTlas && s->insts.size() >= 2)
  {
    const int st = build_tlas(s);
    if (st != HRT_OK)
    {
      cudaStreamSynchronize(ctx->stream);
      free_geom(s->tlas);
      return st;
    }
  }
  if (s->dInst) cudaFree(s->dInst);
  s->dInst = nullptr;
  s->nInstDev = (uint32_t)d.size();
  s->single = d.size() == 1 && d[0].identity && d[0].valid && s->tlas.nTris == 0;
  if (s->single)
  {
    s->singleDesc = d[0];
    const Geom& g0 = s->geoms[s->insts[0].geomId];
    s->singleNodeBytes = s->layout == HRT_LAYOUT_BVH2 ? sizeof(PairRec) * (size_t)(g0.nLeaves > 1 ? g0.nLeaves - 1 : 1)
                                                      : (s->layout == HRT_LAYOUT_BVH4_F32 ? sizeof(Node4F32)
                                                                                         : sizeof(Node4F16)) *
                                                            (size_t)g0.nNodes4;
  }
  if (!d.empty())
  {
    HRT_CUDA(ctx, cudaMalloc((void**)&s->dInst, sizeof(InstanceDesc) * d.size()));
    HRT_CUDA(ctx, cudaMemcpy(s->dInst, d.data(), sizeof(InstanceDesc) * d.size(), cudaMemcpyHostToDevice));
  }
  s->committed = true;
  return HRT_OK;
}

int hrt_query_nearest(hrt_scene* s, const float* rays, uint64_t n, hrt_hit* hits, void* stream)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  return launch_query(s, 0, rays, n, hits, 0, (cudaStream_t)stream);
}

int hrt_query_any(hrt_scene* s, const float* rays, uint64_t n, uint8_t* out, void* stream)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  return launch_query(s, 1, rays, n, out, 0, (cudaStream_t)stream);
}

// Reads (after the work on `cs`) and clears the scene's device-side check
// word: the step budget, the stack bound, index checks of the traversals.
static int read_device_check(hrt_scene* s, cudaStream_t cs)
{
  hrt_context* ctx = s->ctx;
  uint32_t ew[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  HRT_CUDA(ctx, cudaMemcpyAsync(ew, s->dError, sizeof(ew), cudaMemcpyDeviceToHost, cs));
  HRT_CUDA(ctx, cudaStreamSynchronize(cs));
  const uint32_t err = ew[0];
  if (!err) return HRT_OK;
  cudaMemsetAsync(s->dError, 0, sizeof(ew), cs);
  cudaStreamSynchronize(cs);
  if (err & kErrStepBudget)
  {
    char msg[200];
    std::snprintf(msg, sizeof(msg), "a ray exceeded the traversal step budget (ray %u, ref 0x%08x, stack depth %d)",
                  ew[2], ew[3], (int)ew[4]);
    return fail(ctx, HRT_ERR_DEVICE_CHECK, msg);
  }
  if (err & kErrStack) return fail(ctx, HRT_ERR_DEVICE_CHECK, "traversal stack bound exceeded");
  return fail(ctx, HRT_ERR_DEVICE_CHECK, "device-side check failed during a query");
}

static int query_host(hrt_scene* s, int kind, const float* rays, uint64_t n, void* out)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  if (n == 0) return HRT_OK;
  if (!rays || !out) return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "null ray or output pointer");
  std::lock_guard<std::mutex> g(s->mu);
  hrt_context* ctx = s->ctx;
  cudaSetDevice(ctx->device);
  cudaStream_t cs = ctx->stream;
  int st = HRT_OK;
  // Page-locked host arrays are mapped into the GPU's address space: the
  // traversal reads such rays in place over the host link and writes the
  // results in place too.  Where the device translates through the host's
  // page tables, pageable rays are read in place as well (results into
  // pageable memory still come back by copy).  Nearest hits in place come from the one-thread-per-
  // ray kernel, whose warps write 32 consecutive hits at once (the persistent
  // pool writes each hit when its ray ends, scattered 32-byte writes that the
  // link serves poorly).  Other host memory (or arrays that are not 16-byte
  // aligned) goes through the staging buffers.
  const float* mappedRays = aligned_to(rays, 16) ? static_cast<const float*>(mapped_host(rays, true)) : nullptr;
  void* mappedOut = kind == 1 || aligned_to(out, 16) ? mapped_host(out) : nullptr;
  const bool inPlace = mappedRays && mappedOut;
  if (inPlace)
  {
    QuerySegments q;
    TraceConfig grid = s->cfg[kind];
    if (kind == 0)
    {
      grid.persistent = 0;
      grid.threadsPerBlock = 128;
      q.config = &grid;
    }
    st = launch_query(s, kind, mappedRays, n, mappedOut, 0, cs, q);
    if (st != HRT_OK) return st;
  }
  else if ((st = ensure_stage(s, n)) != HRT_OK)
    return st;
  // Otherwise large batches are cut into chunks that cycle over the scene's
  // pipeline streams, so that one chunk's upload, another's traversal and a
  // third's download overlap (the copy engines and the SMs work at once).
  // Each chunk has its own part of the staging buffers; results do not depend
  // on the cut.
  constexpr uint64_t kMinChunk = 1u << 17, kChunks = 8;
  const uint64_t chunk = n < 2 * kMinChunk ? n : std::max<uint64_t>(kMinChunk, (n + kChunks - 1) / kChunks);
  const size_t outSize = kind == 0 ? sizeof(hrt_hit) : 1;
  const int nPipe = (chunk == n || inPlace) ? 1 : 3;
  if (nPipe > 1)
    for (cudaStream_t& p : s->pipe)
      if (!p) HRT_CUDA(ctx, cudaStreamCreateWithFlags(&p, cudaStreamNonBlocking));
  for (uint64_t c0 = 0, k = 0; c0 < n && !inPlace; c0 += chunk, k++)
  {
    const uint64_t len = std::min(chunk, n - c0);
    cudaStream_t ps = nPipe > 1 ? s->pipe[k % nPipe] : cs;
    const float* src = rays + 8 * c0;
    float* dRays = static_cast<float*>(s->stageRays) + 8 * c0;
    uint8_t* dOut = static_cast<uint8_t*>(s->stageOut) + outSize * c0;
    if (mappedRays)
      st = launch_query(s, kind, mappedRays + 8 * c0, len, dOut, 0, ps);
    else
    {
      HRT_CUDA(ctx, cudaMemcpyAsync(dRays, src, 32 * len, cudaMemcpyHostToDevice, ps));
      st = launch_query(s, kind, dRays, len, dOut, 0, ps);
    }
    if (st != HRT_OK)
    {
      for (int p = 0; p < nPipe && nPipe > 1; p++) cudaStreamSynchronize(s->pipe[p]);
      return st;
    }
    HRT_CUDA(ctx, cudaMemcpyAsync(static_cast<uint8_t*>(out) + outSize * c0, dOut, outSize * len,
                                  cudaMemcpyDeviceToHost, ps));
  }
  if (nPipe > 1)
    for (int p = 0; p < nPipe; p++) HRT_CUDA(ctx, cudaStreamSynchronize(s->pipe[p]));
  return read_device_check(s, cs);
}

// Asynchronous host-pointer query: page-locked (16-byte aligned) rays are read
// in place and page-locked results written in place; everything else goes
// through stream-ordered device allocations and copies on `st`.
static int query_host_async(hrt_scene* s, int kind, const float* rays, uint64_t n, void* out, cudaStream_t st)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  if (n == 0) return HRT_OK;
  if (!rays || !out) return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "null ray or output pointer");
  hrt_context* ctx = s->ctx;
  cudaSetDevice(ctx->device);
  const float* mappedRays = aligned_to(rays, 16) ? static_cast<const float*>(mapped_host(rays, true)) : nullptr;
  void* mappedOut = kind == 1 || aligned_to(out, 16) ? mapped_host(out) : nullptr;
  const size_t outSize = kind == 0 ? sizeof(hrt_hit) : 1;
  float* dRays = nullptr;
  void* dOut = nullptr;
  if (!mappedRays)
  {
    HRT_CUDA(ctx, cudaMallocAsync((void**)&dRays, 32 * n, st));
    HRT_CUDA(ctx, cudaMemcpyAsync(dRays, rays, 32 * n, cudaMemcpyHostToDevice, st));
  }
  if (!mappedOut) HRT_CUDA(ctx, cudaMallocAsync(&dOut, outSize * n, st));
  QuerySegments q;
  TraceConfig grid = s->cfg[kind];
  if (kind == 0 && mappedOut)
  {
    grid.persistent = 0;  // hits written in place: see query_host
    grid.threadsPerBlock = 128;
    q.config = &grid;
  }
  int r = launch_query(s, kind, mappedRays ? mappedRays : dRays, n, mappedOut ? mappedOut : dOut, 0, st, q);
  cudaError_t e = cudaSuccess;
  if (r == HRT_OK && dOut) e = cudaMemcpyAsync(out, dOut, outSize * n, cudaMemcpyDeviceToHost, st);
  if (dRays) cudaFreeAsync(dRays, st);
  if (dOut) cudaFreeAsync(dOut, st);
  if (r == HRT_OK && e != cudaSuccess) r = cuda_fail(ctx, e, "result copy");
  return r;
}

int hrt_query_nearest_host(hrt_scene* s, const float* rays, uint64_t n, hrt_hit* hits)
{
  return query_host(s, 0, rays, n, hits);
}

int hrt_query_any_host(hrt_scene* s, const float* rays, uint64_t n, uint8_t* out) { return query_host(s, 1, rays, n, out); }

int hrt_query_nearest_host_async(hrt_scene* s, const float* rays, uint64_t n, hrt_hit* hits, void* stream)
{
  return query_host_async(s, 0, rays, n, hits, (cudaStream_t)stream);
}

int hrt_query_any_host_async(hrt_scene* s, const float* rays, uint64_t n, uint8_t* out, void* stream)
{
  return query_host_async(s, 1, rays, n, out, (cudaStream_t)stream);
}

int hrt_scene_check(hrt_scene* s)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(s->ctx->device);
  return read_device_check(s, s->ctx->stream);
}

int hrt_query_counters(hrt_scene* s, int kind, const float* rays, uint64_t n, uint64_t counters[2], void* stream)
{
  if (!s || !counters || (kind != 0 && kind != 1)) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = s->ctx;
  cudaStream_t cs = (cudaStream_t)stream;
  void* out = nullptr;
  HRT_CUDA(ctx, cudaMallocAsync(&out, kind == 0 ? sizeof(hrt_hit) * (n ? n : 1) : (n ? n : 1), cs));
  HRT_CUDA(ctx, cudaMemsetAsync(s->dCounters, 0, 2 * sizeof(unsigned long long), cs));
  HRT_CUDA(ctx, cudaMemsetAsync(s->dError, 0, sizeof(uint32_t), cs));
  int st = launch_query(s, kind, rays, n, out, 1, cs);
  unsigned long long c[2] = {0, 0};
  uint32_t err = 0;
  HRT_CUDA(ctx, cudaMemcpyAsync(c, s->dCounters, sizeof(c), cudaMemcpyDeviceToHost, cs));
  HRT_CUDA(ctx, cudaMemcpyAsync(&err, s->dError, sizeof(err), cudaMemcpyDeviceToHost, cs));
  HRT_CUDA(ctx, cudaFreeAsync(out, cs));
  HRT_CUDA(ctx, cudaStreamSynchronize(cs));
  if (st != HRT_OK) return st;
  counters[0] = c[0];
  counters[1] = c[1];
  if (err & kErrStack) return fail(ctx, HRT_ERR_DEVICE_CHECK, "traversal stack bound exceeded");
  return HRT_OK;
}

int hrt_get_geom_num(const hrt_scene* s, uint32_t* out)
{
  if (!s || !out) return HRT_ERR_INVALID_ARGUMENT;
  *out = (uint32_t)s->geoms.size();
  return HRT_OK;
}

int hrt_get_inst_num(const hrt_scene* s, uint32_t* out)
{
  if (!s || !out) return HRT_ERR_INVALID_ARGUMENT;
  *out = (uint32_t)s->insts.size();
  return HRT_OK;
}

int hrt_get_geom_boxes(const hrt_scene* s, float* boxes, uint32_t capacity)
{
  if (!s || (!boxes && capacity)) return HRT_ERR_INVALID_ARGUMENT;
  const uint32_t n = (uint32_t)s->geoms.size();
  for (uint32_t i = 0; i < n && i < capacity; i++) std::memcpy(boxes + 8 * i, s->geoms[i].box, 8 * sizeof(float));
  return HRT_OK;
}

int hrt_geom_info(const hrt_scene* s, uint32_t geomId, uint64_t out[4], float* build_ms)
{
  if (!s || !out || geomId >= s->geoms.size()) return HRT_ERR_INVALID_ARGUMENT;
  const Geom& g = s->geoms[geomId];
  out[0] = g.nTris;
  out[1] = g.nLeaves;
  out[2] = (s->layout == HRT_LAYOUT_BVH2) ? (g.nLeaves > 1 ? g.nLeaves - 1 : (g.nTris ? 1 : 0)) : g.nNodes4;
  out[3] = g.bytes;
  if (build_ms) *build_ms = g.buildMs;
  return HRT_OK;
}

int hrt_geom_export(const hrt_scene* s, uint32_t geomId, int what, void* dst, uint64_t capacityBytes, uint64_t* sizeBytes)
{
  if (!s || geomId >= s->geoms.size()) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = s->ctx;
  const Geom& g = s->geoms[geomId];
  const uint64_t N = g.nTris, L = g.nLeaves, nLR = L ? 2 * L - 1 : 0;
  uint64_t size = 0;
  switch (what)
  {
    case HRT_EXPORT_SCENE_BOX: size = 12 * sizeof(float); break;
    case HRT_EXPORT_MORTON_SORTED:
    case HRT_EXPORT_MORTON_UNSORTED: size = 8 * N; break;
    case HRT_EXPORT_COMPRESSED:
    case HRT_EXPORT_RUN_STARTS: size = 4 * L; break;
    case HRT_EXPORT_LR_NODES: size = 32 * nLR; break;
    case HRT_EXPORT_LR_COUNTS: size = 4 * nLR; break;
    case HRT_EXPORT_PRIM_INDICES: size = 4 * N; break;
    case HRT_EXPORT_SORTED_INDICES: size = 12 * N; break;
    case HRT_EXPORT_NODES4:
      size = (uint64_t)g.nNodes4 * (s->layout == HRT_LAYOUT_BVH4_F32 ? sizeof(Node4F32) : sizeof(Node4F16));
      break;
    case HRT_EXPORT_PAIR_RECORDS: size = g.recs ? sizeof(PairRec) * (L > 1 ? L - 1 : (L ? 1 : 0)) : 0; break;
    default: return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "unknown export id");
  }
  if (sizeBytes) *sizeBytes = size;
  if (!dst) return HRT_OK;
  if (capacityBytes < size) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "export buffer too small");
  if (size == 0) return HRT_OK;
  cudaSetDevice(ctx->device);
  switch (what)
  {
    case HRT_EXPORT_SCENE_BOX:
      std::memcpy(dst, g.host.bmin, 12 * sizeof(float));
      return HRT_OK;
    case HRT_EXPORT_MORTON_SORTED:
    case HRT_EXPORT_MORTON_UNSORTED:
    {
      std::vector<uint32_t> k(N), v(N);
      const uint32_t* src = what == HRT_EXPORT_MORTON_SORTED ? g.keys : g.keysUnsorted;
      HRT_CUDA(ctx, cudaMemcpy(k.data(), src, 4 * N, cudaMemcpyDeviceToHost));
      if (what == HRT_EXPORT_MORTON_SORTED) HRT_CUDA(ctx, cudaMemcpy(v.data(), g.vals, 4 * N, cudaMemcpyDeviceToHost));
      else
        for (uint64_t i = 0; i < N; i++) v[i] = (uint32_t)i;
      uint32_t* o = (uint32_t*)dst;
      for (uint64_t i = 0; i < N; i++)
      {
        o[2 * i] = k[i];
        o[2 * i + 1] = v[i];
      }
      return HRT_OK;
    }
    case HRT_EXPORT_COMPRESSED: HRT_CUDA(ctx, cudaMemcpy(dst, g.compressed, size, cudaMemcpyDeviceToHost)); return HRT_OK;
    case HRT_EXPORT_RUN_STARTS: HRT_CUDA(ctx, cudaMemcpy(dst, g.runStarts, size, cudaMemcpyDeviceToHost)); return HRT_OK;
    case HRT_EXPORT_LR_NODES: HRT_CUDA(ctx, cudaMemcpy(dst, g.lr, size, cudaMemcpyDeviceToHost)); return HRT_OK;
    case HRT_EXPORT_LR_COUNTS: HRT_CUDA(ctx, cudaMemcpy(dst, g.lrCount, size, cudaMemcpyDeviceToHost)); return HRT_OK;
    case HRT_EXPORT_PRIM_INDICES: HRT_CUDA(ctx, cudaMemcpy(dst, g.vals, size, cudaMemcpyDeviceToHost)); return HRT_OK;
    case HRT_EXPORT_SORTED_INDICES: HRT_CUDA(ctx, cudaMemcpy(dst, g.sortedIdx, size, cudaMemcpyDeviceToHost)); return HRT_OK;
    case HRT_EXPORT_NODES4: HRT_CUDA(ctx, cudaMemcpy(dst, g.nodes4, size, cudaMemcpyDeviceToHost)); return HRT_OK;
    case HRT_EXPORT_PAIR_RECORDS: HRT_CUDA(ctx, cudaMemcpy(dst, g.recs, size, cudaMemcpyDeviceToHost)); return HRT_OK;
    default: break;
  }
  return HRT_ERR_INVALID_ARGUMENT;
}

int hrt_scene_set_layout(hrt_scene* s, int layout)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  if (layout < HRT_LAYOUT_BVH2 || layout > HRT_LAYOUT_BVH4_Q8) return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "unknown layout");
  std::lock_guard<std::mutex> g(s->mu);
  if (!s->geoms.empty()) return fail(s->ctx, HRT_ERR_STATE, "the layout is chosen before the first geometry is added");
  s->layout = layout;
  return HRT_OK;
}

int hrt_scene_set_option(hrt_scene* s, int option, int value)
{
  if (!s) return HRT_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> g(s->mu);
  switch (option)
  {
    case HRT_OPTION_BVH4_MERGE:
      if (value < 0 || value > 64) return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "BVH4 merge value out of range");
      s->bvh4Merge = value;
      return HRT_OK;
    case HRT_OPTION_TLAS:
      if (value != 0 && value != 1) return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "TLAS option is 0 or 1");
      s->useTlas = value;
      s->committed = false;
      return HRT_OK;
    case HRT_OPTION_L2_PERSIST:
    {
      if (value < 0 || value > 4096) return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "L2 persisting size out of range");
      int maxPersist = 0;
      cudaSetDevice(s->ctx->device);
      if (cudaDeviceGetAttribute(&maxPersist, cudaDevAttrMaxPersistingL2CacheSize, s->ctx->device) != cudaSuccess)
        return fail(s->ctx, HRT_ERR_CUDA, "cannot read the persisting L2 capacity");
      if (value > 0 && maxPersist == 0) return fail(s->ctx, HRT_ERR_UNSUPPORTED, "device has no persisting L2");
      // the set-aside is a limit of the process's context on this device
      const size_t bytes = std::min<size_t>((size_t)value << 20, (size_t)maxPersist);
      if ((value > 0 || s->l2PersistMB > 0) && cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, bytes) != cudaSuccess)
        return fail(s->ctx, HRT_ERR_CUDA, "cannot set the persisting L2 size");
      if (value == 0 && s->l2PersistMB > 0) cudaCtxResetPersistingL2Cache();  // persisting lines back to normal
      s->l2PersistMB = value;
      return HRT_OK;
    }
    case HRT_OPTION_MORTON_FRAME:
      if (value != HRT_MORTON_PER_AXIS && value != HRT_MORTON_CUBIC)
        return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "unknown Morton frame");
      s->mortonFrame = value;
      return HRT_OK;
    case HRT_OPTION_BVH4_COLLAPSE:
      if (value != HRT_BVH4_COLLAPSE_EVEN_DEPTH && value != HRT_BVH4_COLLAPSE_LARGEST_FIRST)
        return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "unknown BVH4 collapse rule");
      s->bvh4Collapse = value;
      return HRT_OK;
    case HRT_OPTION_TRIANGLE_TEST:
      if (value != HRT_TRI_MOLLER_TRUMBORE && value != HRT_TRI_WATERTIGHT)
        return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "unknown triangle test");
      if (!s->geoms.empty())
        return fail(s->ctx, HRT_ERR_STATE, "the triangle test is chosen before the first geometry is added");
      s->triTest = value;
      return HRT_OK;
    default: return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "unknown option");
  }
}

int hrt_scene_get_layout(const hrt_scene* s, int* layout)
{
  if (!s || !layout) return HRT_ERR_INVALID_ARGUMENT;
  *layout = s->layout;
  return HRT_OK;
}

int hrt_scene_set_trace_config(hrt_scene* s, int kind, const hrt_trace_config* c)
{
  if (!s || !c || (kind != 0 && kind != 1)) return HRT_ERR_INVALID_ARGUMENT;
  if ((c->threadsPerBlock != 64 && c->threadsPerBlock != 128 && c->threadsPerBlock != 256) ||
      (c->persistent != 0 && c->persistent != 1) || c->stepsPerRefill < 1 || c->stepsPerRefill > 1024 ||
      c->refillLanes < 1 || c->refillLanes > 32 || c->stackEntries < 0 || c->stackEntries > HRT_MAX_STACK_ENTRIES ||
      c->imageWidth < 0)
    return fail(s->ctx, HRT_ERR_INVALID_ARGUMENT, "trace config out of range");
  std::lock_guard<std::mutex> g(s->mu);
  s->cfg[kind].threadsPerBlock = c->threadsPerBlock;
  s->cfg[kind].persistent = c->persistent;
  s->cfg[kind].stepsPerRefill = c->stepsPerRefill;
  s->cfg[kind].refillLanes = c->refillLanes;
  s->cfg[kind].stackEntries = c->stackEntries;
  s->cfg[kind].imageWidth = c->imageWidth;
  return HRT_OK;
}

int hrt_scene_get_trace_config(const hrt_scene* s, int kind, hrt_trace_config* c)
{
  if (!s || !c || (kind != 0 && kind != 1)) return HRT_ERR_INVALID_ARGUMENT;
  c->threadsPerBlock = s->cfg[kind].threadsPerBlock;
  c->persistent = s->cfg[kind].persistent;
  c->stepsPerRefill = s->cfg[kind].stepsPerRefill;
  c->refillLanes = s->cfg[kind].refillLanes;
  c->stackEntries = s->cfg[kind].stackEntries;
  c->imageWidth = s->cfg[kind].imageWidth;
  return HRT_OK;
}

int hrt_query_multi(hrt_scene* s, const hrt_query_desc* q, void* stream)
{
  if (!s || !q || (q->kind != 0 && q->kind != 1)) return HRT_ERR_INVALID_ARGUMENT;
  QuerySegments sg;
  sg.rayOffsets = q->rayOffsets;
  sg.segInst = q->segInst;
  sg.nSeg = q->nSeg;
  return launch_query(s, q->kind, q->rays, q->n, q->out, 0, (cudaStream_t)stream, sg);
}

}  // extern "C"

struct hrt_graph
{
  hrt_scene*      scene = nullptr;
  cudaGraph_t     graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned int*   counters = nullptr;  // one work counter per captured query
};

extern "C" {

int hrt_graph_create(hrt_scene* s, const hrt_query_desc* queries, uint32_t count, hrt_graph** out)
{
  if (!s || !out || (count && !queries)) return HRT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  hrt_context* ctx = s->ctx;
  if (count == 0) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "a graph needs at least one query");
  for (uint32_t i = 0; i < count; i++)
    if (queries[i].kind != 0 && queries[i].kind != 1) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "unknown query kind");
  if (!s->committed) return fail(ctx, HRT_ERR_STATE, "graph capture before hrt_commit_scene");
  cudaSetDevice(ctx->device);
  hrt_graph* g = new hrt_graph();
  g->scene = s;
  cudaStream_t cs = nullptr;
  auto cleanup = [&](int status) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->counters) cudaFree(g->counters);
    if (cs) cudaStreamDestroy(cs);
    delete g;
    return status;
  };
  cudaError_t e = cudaMalloc((void**)&g->counters, sizeof(unsigned int) * count);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "graph counters"));
  e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "capture stream"));
  // the relaxed mode lets the launcher query occupancy while capturing
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "cudaStreamBeginCapture"));
  int st = HRT_OK;
  for (uint32_t i = 0; i < count && st == HRT_OK; i++)
  {
    QuerySegments sg;
    sg.rayOffsets = queries[i].rayOffsets;
    sg.segInst = queries[i].segInst;
    sg.nSeg = queries[i].nSeg;
    sg.counter = g->counters + i;
    st = launch_query(s, queries[i].kind, queries[i].rays, queries[i].n, queries[i].out, 0, cs, sg);
  }
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(cs, &graph);
  g->graph = graph;
  if (st != HRT_OK) return cleanup(st);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "cudaStreamEndCapture"));
  e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "cudaGraphInstantiate"));
  cudaStreamDestroy(cs);
  *out = g;
  return HRT_OK;
}

int hrt_graph_launch(hrt_graph* g, void* stream)
{
  if (!g) return HRT_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(g->scene->ctx, e, "cudaGraphLaunch");
  return HRT_OK;
}

int hrt_graph_destroy(hrt_graph* g)
{
  if (!g) return HRT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(g->scene->ctx->device);
  cudaDeviceSynchronize();
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->counters) cudaFree(g->counters);
  delete g;
  return HRT_OK;
}

int hrt_scene_autotune(hrt_scene* s, const hrt_query_desc* q, int repeats, hrt_trace_config* best, float* bestMs)
{
  if (!s || !q || (q->kind != 0 && q->kind != 1)) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = s->ctx;
  if (repeats < 1 || repeats > 1000) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "repeats out of range");
  cudaSetDevice(ctx->device);
  std::vector<TraceConfig> grid;
  for (int tpb : {64, 128, 256})
  {
    TraceConfig c;
    c.imageWidth = s->cfg[q->kind].imageWidth;  // a property of the rays, kept
    c.threadsPerBlock = tpb;
    c.persistent = 0;
    grid.push_back(c);
    for (int steps : {4, 8, 16, 32, 64})
      for (int lanes : {2, 4, 8, 16, 24, 28, 32})
      {
        c.persistent = 1;
        c.stepsPerRefill = steps;
        c.refillLanes = lanes;
        grid.push_back(c);
      }
  }
  const TraceConfig saved = s->cfg[q->kind];
  cudaStream_t cs = ctx->stream;
  cudaEvent_t e0, e1;
  HRT_CUDA(ctx, cudaEventCreate(&e0));
  HRT_CUDA(ctx, cudaEventCreate(&e1));
  QuerySegments sg;
  sg.rayOffsets = q->rayOffsets;
  sg.segInst = q->segInst;
  sg.nSeg = q->nSeg;
  float bestT = INFINITY;
  TraceConfig bestC = saved;
  int st = HRT_OK;
  for (const TraceConfig& c : grid)
  {
    s->cfg[q->kind] = c;
    st = launch_query(s, q->kind, q->rays, q->n, q->out, 0, cs, sg);  // warm-up
    if (st != HRT_OK) break;
    cudaEventRecord(e0, cs);
    for (int r = 0; r < repeats && st == HRT_OK; r++) st = launch_query(s, q->kind, q->rays, q->n, q->out, 0, cs, sg);
    cudaEventRecord(e1, cs);
    if (st != HRT_OK) break;
    if (cudaEventSynchronize(e1) != cudaSuccess)
    {
      st = cuda_fail(ctx, cudaGetLastError(), "autotune timing");
      break;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= (float)repeats;
    if (ms < bestT)
    {
      bestT = ms;
      bestC = c;
    }
  }
  // second stage: the short stack's size under the best launch shape
  // (entries beyond it spill to local memory; 64 covers every depth bound of
  // a single-level tree)
  if (st == HRT_OK)
  {
    const TraceConfig shape = bestC;
    for (int entries : {16, 24, 32, 48, 64})
    {
      TraceConfig c = shape;
      c.stackEntries = entries;
      s->cfg[q->kind] = c;
      st = launch_query(s, q->kind, q->rays, q->n, q->out, 0, cs, sg);  // warm-up
      if (st != HRT_OK) break;
      cudaEventRecord(e0, cs);
      for (int r = 0; r < repeats && st == HRT_OK; r++) st = launch_query(s, q->kind, q->rays, q->n, q->out, 0, cs, sg);
      cudaEventRecord(e1, cs);
      if (st != HRT_OK) break;
      if (cudaEventSynchronize(e1) != cudaSuccess)
      {
        st = cuda_fail(ctx, cudaGetLastError(), "autotune timing");
        break;
      }
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= (float)repeats;
      if (ms < bestT)
      {
        bestT = ms;
        bestC = c;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s->cfg[q->kind] = (st == HRT_OK) ? bestC : saved;
  if (st != HRT_OK) return st;
  uint32_t err = 0;
  HRT_CUDA(ctx, cudaMemcpy(&err, s->dError, sizeof(err), cudaMemcpyDeviceToHost));
  if (err)
  {
    cudaMemset(s->dError, 0, 8 * sizeof(uint32_t));
    return fail(ctx, HRT_ERR_DEVICE_CHECK, "device-side check failed during autotuning");
  }
  if (best)
  {
    best->threadsPerBlock = bestC.threadsPerBlock;
    best->persistent = bestC.persistent;
    best->stepsPerRefill = bestC.stepsPerRefill;
    best->refillLanes = bestC.refillLanes;
    best->stackEntries = bestC.stackEntries;
    best->imageWidth = bestC.imageWidth;
  }
  if (bestMs) *bestMs = bestT;
  return HRT_OK;
}

int hrt_host_alloc(uint64_t bytes, void** out)
{
  if (!out) return HRT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) return HRT_ERR_OUT_OF_MEMORY;
  return HRT_OK;
}

int hrt_host_free(void* p)
{
  if (p && cudaFreeHost(p) != cudaSuccess) return HRT_ERR_CUDA;
  return HRT_OK;
}

}  // extern "C"
