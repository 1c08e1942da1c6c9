// On-disk formats: HeavyRT's VSGF meshes and the engine's own BVH blobs.
//
// VSGF (examples/loader/cmesh.cpp:80-173): a 24-byte header {u64 file size,
// u32 vertices, u32 indices, u32 materials, u32 flags}, then float4 positions,
// float4 normals (absent with flag 8), float4 tangents (present with flag 1),
// float2 texture coordinates, u32 indices and one u32 material id per
// triangle.
//
// BVH blob ("HRTBVH02"): everything a built geometry keeps on the device
// (vertices, build stage arrays, and the binary pair records or the 4-wide
// nodes its layout traverses), so that a
// geometry can be restored by copies alone, without a build: a warm start for
// a server's resident scenes.  Blobs are tied to the layout they were built
// with.
#include <cstdio>
#include <cstring>
#include <vector>

#include "hrt_internal.cuh"

using namespace hrt;
using namespace hrt::api;

namespace
{

struct VsgfHeader
{
  uint64_t fileSize;
  uint32_t vertices, indices, materials, flags;
};
static_assert(sizeof(VsgfHeader) == 24, "VSGF header is 24 bytes");

constexpr uint32_t kHasTangent = 1, kHasNoNormals = 8;

struct File
{
  FILE* f = nullptr;
  explicit File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
  ~File()
  {
    if (f) std::fclose(f);
  }
};

bool read_vsgf_header(FILE* f, VsgfHeader& h, uint64_t& actual)
{
  if (std::fseek(f, 0, SEEK_END) != 0) return false;
  const long end = std::ftell(f);
  if (end < (long)sizeof(VsgfHeader) || std::fseek(f, 0, SEEK_SET) != 0) return false;
  actual = (uint64_t)end;
  if (std::fread(&h, sizeof(h), 1, f) != 1) return false;
  const uint64_t V = h.vertices;
  const uint64_t need = sizeof(VsgfHeader) + 16 * V * (1 + ((h.flags & kHasNoNormals) ? 0 : 1) + ((h.flags & kHasTangent) ? 1 : 0)) +
                        8 * V + 4 * (uint64_t)h.indices + 4 * ((uint64_t)h.indices / 3);
  return h.indices % 3 == 0 && actual >= need;
}

// ---------------------------------------------------------------- BVH blobs
constexpr char kBlobMagic[8] = {'H', 'R', 'T', 'B', 'V', 'H', '0', '2'};

struct BlobHeader
{
  char     magic[8];
  uint32_t layout, merge;
  uint32_t nTris, nVerts, nLeaves, nNodes4;
  BuildParams params;
};

// Device arrays of a geometry in blob order, with their byte sizes.
struct Part
{
  void*  ptr;
  size_t bytes;
};

std::vector<Part> parts(Geom& g, int layout)
{
  const size_t N = g.nTris, L = g.nLeaves, V = g.nVerts, nLR = L ? 2 * L - 1 : 0;
  const size_t nodeBytes = layout == HRT_LAYOUT_BVH4_F32 ? sizeof(Node4F32) : sizeof(Node4F16);
  std::vector<Part> p = {{g.verts, 16 * V},
                         {g.keys, 4 * N},
                         {g.vals, 4 * N},
                         {g.keysUnsorted, 4 * N},
                         {g.compressed, 4 * L},
                         {g.runStarts, 4 * L},
                         {g.lr, sizeof(BVHNode32) * nLR},
                         {g.lrCount, 4 * nLR},
                         {g.tris, sizeof(TriRec) * N},
                         {g.sortedIdx, 12 * N}};
  if (layout == HRT_LAYOUT_BVH2) p.push_back({g.recs, sizeof(PairRec) * (L > 1 ? L - 1 : 1)});
  else p.push_back({g.nodes4, nodeBytes * g.nNodes4});
  return p;
}

}  // namespace

extern "C" {

int hrt_vsgf_info(const char* path, uint64_t* nVert, uint64_t* nIdx, uint32_t* flags)
{
  if (!path) return HRT_ERR_INVALID_ARGUMENT;
  File f(path, "rb");
  if (!f.f) return HRT_ERR_INVALID_ARGUMENT;
  VsgfHeader h;
  uint64_t actual = 0;
  if (!read_vsgf_header(f.f, h, actual)) return HRT_ERR_INVALID_ARGUMENT;
  if (nVert) *nVert = h.vertices;
  if (nIdx) *nIdx = h.indices;
  if (flags) *flags = h.flags;
  return HRT_OK;
}

int hrt_vsgf_read(const char* path, float* vpos4, uint32_t* idx, float* norm4)
{
  if (!path || !vpos4 || !idx) return HRT_ERR_INVALID_ARGUMENT;
  File f(path, "rb");
  if (!f.f) return HRT_ERR_INVALID_ARGUMENT;
  VsgfHeader h;
  uint64_t actual = 0;
  if (!read_vsgf_header(f.f, h, actual)) return HRT_ERR_INVALID_ARGUMENT;
  const size_t V = h.vertices;
  if (std::fread(vpos4, 16, V, f.f) != V) return HRT_ERR_INVALID_ARGUMENT;
  if (!(h.flags & kHasNoNormals))
  {
    if (norm4)
    {
      if (std::fread(norm4, 16, V, f.f) != V) return HRT_ERR_INVALID_ARGUMENT;
    }
    else if (std::fseek(f.f, (long)(16 * V), SEEK_CUR) != 0)
      return HRT_ERR_INVALID_ARGUMENT;
  }
  else if (norm4)
    std::memset(norm4, 0, 16 * V);
  const long skip = (long)(((h.flags & kHasTangent) ? 16 * V : 0) + 8 * V);  // tangents, texture coordinates
  if (std::fseek(f.f, skip, SEEK_CUR) != 0) return HRT_ERR_INVALID_ARGUMENT;
  if (std::fread(idx, 4, h.indices, f.f) != h.indices) return HRT_ERR_INVALID_ARGUMENT;
  return HRT_OK;
}

int hrt_vsgf_write(const char* path, const float* vpos4, uint64_t nVert, const uint32_t* idx, uint64_t nIdx)
{
  if (!path || (nVert && !vpos4) || (nIdx && !idx) || nIdx % 3 != 0 || nVert > 0xFFFFFFFFull || nIdx > 0xFFFFFFFFull)
    return HRT_ERR_INVALID_ARGUMENT;
  File f(path, "wb");
  if (!f.f) return HRT_ERR_INVALID_ARGUMENT;
  VsgfHeader h;
  h.vertices = (uint32_t)nVert;
  h.indices = (uint32_t)nIdx;
  h.materials = 0;
  h.flags = kHasNoNormals;
  h.fileSize = sizeof(h) + 16 * nVert + 8 * nVert + 4 * nIdx + 4 * (nIdx / 3);
  const std::vector<float> tex(2 * nVert, 0.0f);
  const std::vector<uint32_t> mat(nIdx / 3, 0u);
  const bool ok = std::fwrite(&h, sizeof(h), 1, f.f) == 1 && std::fwrite(vpos4, 16, nVert, f.f) == nVert &&
                  std::fwrite(tex.data(), 8, nVert, f.f) == nVert && std::fwrite(idx, 4, nIdx, f.f) == nIdx &&
                  std::fwrite(mat.data(), 4, nIdx / 3, f.f) == nIdx / 3;
  return ok ? HRT_OK : HRT_ERR_INVALID_ARGUMENT;
}

int hrt_geom_save(const hrt_scene* s, uint32_t geomId, const char* path)
{
  if (!s || !path || geomId >= s->geoms.size()) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = s->ctx;
  Geom g = s->geoms[geomId];
  BlobHeader h;
  std::memcpy(h.magic, kBlobMagic, 8);
  h.layout = (uint32_t)s->layout | ((uint32_t)g.triTest << 8);  // triangle-record form in bits 8..15
  // merge bound in bits 0..7, collapse rule in 8..15, Morton frame in 16..23
  // (what a refit of the restored geometry rebuilds with)
  h.merge = (uint32_t)g.bvh4Merge | ((uint32_t)g.bvh4Collapse << 8) | ((uint32_t)g.mortonFrame << 16);
  h.nTris = g.nTris;
  h.nVerts = g.nVerts;
  h.nLeaves = g.nLeaves;
  h.nNodes4 = g.nNodes4;
  h.params = g.host;
  File f(path, "wb");
  if (!f.f) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
  if (std::fwrite(&h, sizeof(h), 1, f.f) != 1) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "short write");
  if (g.nTris == 0) return HRT_OK;
  cudaSetDevice(ctx->device);
  std::vector<uint8_t> buf;
  for (const Part& p : parts(g, s->layout))
  {
    buf.resize(p.bytes);
    if (p.bytes) HRT_CUDA(ctx, cudaMemcpy(buf.data(), p.ptr, p.bytes, cudaMemcpyDeviceToHost));
    if (p.bytes && std::fwrite(buf.data(), 1, p.bytes, f.f) != p.bytes)
      return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "short write");
  }
  return HRT_OK;
}

int hrt_geom_load(hrt_scene* s, const char* path, uint32_t* geomId)
{
  if (!s || !path) return HRT_ERR_INVALID_ARGUMENT;
  hrt_context* ctx = s->ctx;
  File f(path, "rb");
  if (!f.f) return fail(ctx, HRT_ERR_INVALID_ARGUMENT, std::string("cannot read ") + path);
  BlobHeader h;
  if (std::fread(&h, sizeof(h), 1, f.f) != 1 || std::memcmp(h.magic, kBlobMagic, 6) != 0)
    return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "not a BVH blob");
  if (std::memcmp(h.magic, kBlobMagic, 8) != 0)
    return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "BVH blob of another format version: rebuild the geometry");
  std::lock_guard<std::mutex> lk(s->mu);
  const int triTest = (int)(h.layout >> 8);
  h.layout &= 0xFFu;
  if ((int)h.layout != s->layout) return fail(ctx, HRT_ERR_STATE, "the blob was built for another node layout");
  if (triTest != s->triTest) return fail(ctx, HRT_ERR_STATE, "the blob was built for another triangle test");
  if (h.nTris > HRT_MAX_TRIS_PER_GEOM || h.nLeaves > h.nTris || (h.nTris && !h.nLeaves) ||
      (h.layout != HRT_LAYOUT_BVH2 && h.nTris && !h.nNodes4) || (h.merge & 0xFFu) > 64u ||
      ((h.merge >> 8) & 0xFFu) > (uint32_t)HRT_BVH4_COLLAPSE_LARGEST_FIRST ||
      ((h.merge >> 16) & 0xFFu) > (uint32_t)HRT_MORTON_CUBIC || (h.merge >> 24) != 0u)
    return fail(ctx, HRT_ERR_INVALID_ARGUMENT, "inconsistent BVH blob header");
  cudaSetDevice(ctx->device);
  Geom g;
  g.nTris = h.nTris;
  g.nVerts = h.nVerts;
  g.nLeaves = h.nLeaves;
  g.nNodes4 = h.nNodes4;
  g.bvh4Merge = (int)(h.merge & 0xFFu);
  g.bvh4Collapse = (int)((h.merge >> 8) & 0xFFu);
  g.mortonFrame = (int)((h.merge >> 16) & 0xFFu);
  g.triTest = triTest;
  g.host = h.params;
  for (int c = 0; c < 4; c++)
  {
    g.box[c] = h.nTris ? h.params.bmin[c] : INFINITY;
    g.box[4 + c] = h.nTris ? h.params.bmax[c] : -INFINITY;
  }
  auto bail = [&](int st) {
    cudaDeviceSynchronize();
    free_geom(g);
    return st;
  };
  const size_t N = g.nTris, L = g.nLeaves, V = g.nVerts, nLR = L ? 2 * L - 1 : 0;
  const size_t nodeBytes = h.layout == HRT_LAYOUT_BVH4_F32 ? sizeof(Node4F32) : sizeof(Node4F16);
  struct A
  {
    void** p;
    size_t bytes;
  } allocs[] = {{(void**)&g.verts, 16 * (V ? V : 1)},
                {(void**)&g.params, sizeof(BuildParams)},
                {(void**)&g.keys, 4 * (N ? N : 1)},
                {(void**)&g.vals, 4 * (N ? N : 1)},
                {(void**)&g.keysUnsorted, 4 * (N ? N : 1)},
                {(void**)&g.compressed, 4 * (L ? L : 1)},
                {(void**)&g.runStarts, 4 * (L ? L : 1)},
                {(void**)&g.lr, sizeof(BVHNode32) * (nLR ? nLR : 1)},
                {(void**)&g.lrCount, 4 * (nLR ? nLR : 1)},
                {(void**)&g.tris, sizeof(TriRec) * (N ? N : 1)},
                {(void**)&g.sortedIdx, 12 * (N ? N : 1)},
                {(void**)&g.recs, h.layout == HRT_LAYOUT_BVH2 ? sizeof(PairRec) * (L > 1 ? L - 1 : 1) : 0}};
  for (const A& a : allocs)
  {
    if (a.bytes == 0) continue;
    const cudaError_t e = cudaMalloc(a.p, a.bytes);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "blob allocation"));
    g.bytes += a.bytes;
  }
  if (h.layout != HRT_LAYOUT_BVH2 && N)
  {
    const cudaError_t e = cudaMalloc(&g.nodes4, nodeBytes * g.nNodes4);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "blob allocation"));
    g.bytes += nodeBytes * g.nNodes4;
  }
  if (cudaMemcpy(g.params, &h.params, sizeof(BuildParams), cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(HRT_ERR_CUDA);
  if (N)
  {
    std::vector<uint8_t> buf;
    for (const Part& p : parts(g, (int)h.layout))
    {
      buf.resize(p.bytes);
      if (p.bytes && std::fread(buf.data(), 1, p.bytes, f.f) != p.bytes)
        return bail(fail(ctx, HRT_ERR_INVALID_ARGUMENT, "truncated BVH blob"));
      if (p.bytes && cudaMemcpy(p.ptr, buf.data(), p.bytes, cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(ctx, HRT_ERR_CUDA, "blob upload"));
    }
  }
  s->geoms.push_back(g);
  s->committed = false;
  if (geomId) *geomId = (uint32_t)(s->geoms.size() - 1);
  return HRT_OK;
}

}  // extern "C"
