/*
 * CPU restatement of HeavyRT's hot path: the LBVH build used by BVH2CommonRT
 * with builder "cbvh_lbvh" and the BVH2TraverseC32 nearest/any-hit traversal.
 *
 * TEST INFRASTRUCTURE ONLY.  The engine never links or calls this file: it is
 * the oracle that the tests, the smoke check and the CPU-baseline leg of the
 * benchmark compare the GPU engine with.  Parity of this restatement is pinned
 * against the reference's own sources compiled as a checker (oracle/Makefile.ref
 * + oracle/ref_harness.cpp) and against the golden vectors in tests/golden/.
 *
 * Arithmetic follows the reference operation by operation in IEEE binary32,
 * compiled with -ffp-contract=off.  The vector library the reference uses
 * (LiteMath) is absent from the reference snapshot, so two of its choices are
 * fixed here and in the checker's stand-in header alike: component-wise
 * min(a,b) = a<b ? a : b, max(a,b) = a>b ? a : b; dot = (x*x' + y*y') + z*z'.
 * The slab test uses std::min/std::max (core/raytrace_common.h:67-80), whose
 * semantics are min(a,b) = b<a ? b : a, max(a,b) = a<b ? b : a.
 *
 * One documented deviation: the reference sorts Morton codes with std::sort
 * (core/builders/lbvh.cpp:755), whose order among equal codes is unspecified;
 * the oracle sorts stably (tie-break = original triangle index).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORA_LEAF_BIT   0x80000000u
#define ORA_START_MASK 0x00FFFFFFu
#define ORA_SIZE_MASK  0x7F000000u
#define ORA_STACK_SIZE 80 /* core/raytrace_common.h:34 */

/* BVHNode, 32 bytes (core/builders/cbvh.h:20-26). */
typedef struct
{
  float    boxMin[3];
  uint32_t leftOffset;
  float    boxMax[3];
  uint32_t escapeIndex;
} ora_node;

/* CRT_Hit, 32 bytes (core/CrossRT.h:20-27). */
typedef struct
{
  float    t;
  uint32_t primId, instId, geomId;
  float    coords[4];
} ora_hit;

static inline float fmin_lm(float a, float b) { return (a < b) ? a : b; }   /* LiteMath-style min */
static inline float fmax_lm(float a, float b) { return (a > b) ? a : b; }   /* LiteMath-style max */
static inline float fmin_std(float a, float b) { return (b < a) ? b : a; }  /* std::min */
static inline float fmax_std(float a, float b) { return (a < b) ? b : a; }  /* std::max */

static inline uint32_t pack_offset_and_size(uint32_t start, uint32_t size) /* core/raytrace_common.h:48-51 */
{
  return ORA_LEAF_BIT | ((size << 24) & ORA_SIZE_MASK) | (start & ORA_START_MASK);
}

/* ------------------------------------------------------------------ Morton */

/* SpreadBits / ZIndex3D, core/builders/lbvh.cpp:25-39. */
static inline uint32_t spread_bits(int x, int offset)
{
  x = (x | (x << 10)) & 0x000F801F;
  x = (x | (x << 4)) & 0x00E181C3;
  x = (x | (x << 2)) & 0x03248649;
  x = (x | (x << 2)) & 0x09249249;
  return (uint32_t)x << offset;
}

static inline uint32_t zindex3d(int x, int y, int z) { return spread_bits(x, 0) | spread_bits(y, 1) | spread_bits(z, 2); }

/* Float to int conversion as C++ does it for ZIndex3D(float...) arguments:
 * truncation toward zero (core/builders/lbvh.cpp:282). */
static inline int trunc_to_int(float f) { return (int)f; }

/* Scene AABB over all vertices, core/builders/lbvh.cpp:228-239 (init +-1e10, :53). */
static void aabb_from_vertices(const float* v4, uint32_t nV, float bmin[4], float bmax[4])
{
  for (int c = 0; c < 4; c++) { bmin[c] = 1e10f; bmax[c] = -1e10f; }
  for (uint32_t i = 0; i < nV; i++)
    for (int c = 0; c < 4; c++)
    {
      bmin[c] = fmin_lm(bmin[c], v4[4 * i + c]);
      bmax[c] = fmax_lm(bmax[c], v4[4 * i + c]);
    }
}

/* ZIndexMultCoeff on the biased box, core/builders/lbvh.cpp:41-51 and :263. */
static void zindex_scale(const float bmin[4], const float bmax[4], float scale[4])
{
  for (int c = 0; c < 4; c++)
  {
    const float lo = bmin[c] - 1e-4f;
    const float hi = bmax[c] + 1e-4f;
    float inv = 1.0f / (hi - lo);
    if (c < 3 && fabsf(hi - lo) < 1e-20f) inv = 0.0f;
    scale[c] = 1024.0f * inv;
  }
}

/* kernel1D_EvalMortonCodesFromTriangles, core/builders/lbvh.cpp:259-287. */
static void morton_codes(const float* v4, const uint32_t* idx, uint32_t nTris, const float bmin[4], const float scale[4],
                         uint32_t* pairs /* 2*nTris: (code, triId) */)
{
  for (uint32_t i = 0; i < nTris; i++)
  {
    const float* a = v4 + 4 * (size_t)idx[3 * i + 0];
    const float* b = v4 + 4 * (size_t)idx[3 * i + 1];
    const float* c = v4 + 4 * (size_t)idx[3 * i + 2];
    int q[3];
    for (int k = 0; k < 3; k++)
    {
      float center;
      if (nTris < 256)
        center = 0.33333333f * ((a[k] + b[k]) + c[k]);
      else
      {
        const float mn = fmin_lm(a[k], fmin_lm(b[k], c[k]));
        const float mx = fmax_lm(a[k], fmax_lm(b[k], c[k]));
        center = (mn + mx) * 0.5f;
      }
      q[k] = trunc_to_int(scale[k] * (center - bmin[k]));
    }
    pairs[2 * i + 0] = zindex3d(q[0], q[1], q[2]);
    pairs[2 * i + 1] = i;
  }
}

/* Stable LSD radix sort of (code, id) pairs by code: the same order as
 * std::stable_sort with the comparator of core/builders/lbvh.cpp:755. */
static void sort_pairs_stable(uint32_t* pairs, uint32_t n)
{
  uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)(n ? n : 1));
  uint32_t* src = pairs;
  uint32_t* dst = tmp;
  for (int shift = 0; shift < 32; shift += 8)
  {
    size_t count[257];
    memset(count, 0, sizeof(count));
    for (uint32_t i = 0; i < n; i++) count[((src[2 * i] >> shift) & 0xFF) + 1]++;
    for (int d = 0; d < 256; d++) count[d + 1] += count[d];
    for (uint32_t i = 0; i < n; i++)
    {
      const size_t o = count[(src[2 * i] >> shift) & 0xFF]++;
      dst[2 * o + 0] = src[2 * i + 0];
      dst[2 * o + 1] = src[2 * i + 1];
    }
    uint32_t* t = src; src = dst; dst = t;
  }
  /* four passes: the result is back in `pairs` */
  free(tmp);
}

/* ------------------------------------------------------------------ build */

typedef struct
{
  uint32_t  nTris, nLeaves;
  float     bmin[4], bmax[4], scale[4];
  uint32_t* pairsUnsorted; /* 2*nTris */
  uint32_t* pairsSorted;   /* 2*nTris */
  uint32_t* compressed;    /* nLeaves */
  uint32_t* runStarts;     /* nLeaves */
  ora_node* lr;            /* 2*nLeaves-1, Karras + refit (LR format) */
  uint32_t* lrCount;       /* 2*nLeaves-1, descendant node counts */
  uint32_t* leafIndices;   /* nTris: triangle id at each sorted position */
  ora_node* nodes;         /* peach LEFT_OFFSET layout (cbvh2::BuildBVH output) */
  uint32_t  nNodes;
  uint32_t* indicesSorted; /* 3*nTris, index buffer in sorted order (AppendTreeData) */
  float*    verts;         /* 4*nV, copy of vertex positions with w = 1 */
  uint32_t  nVerts;
  int       status;        /* 0 ok, 1 leaf count above 127 */
} ora_bvh;

/* delta(), core/builders/lbvh.cpp:386-403. */
static inline int karras_delta(const uint32_t* codes, int n, int i, int j)
{
  if (j < 0 || j >= n) return -1;
  const uint32_t x = codes[i] ^ codes[j];
  if (x == 0) return 32;
  int r = 0;
  uint32_t y = x;
  while ((y & 0x80000000u) == 0) { y <<= 1; r++; }
  return r;
}

static inline int isign(int x) { return (x > 0) - (x < 0); }

/* kernel1D_Karras12, core/builders/lbvh.cpp:405-441. */
static void karras12(const uint32_t* codes, int L, ora_node* nodes)
{
  for (int i = 0; i < L - 1; i++)
  {
    const int d = isign(karras_delta(codes, L, i, i + 1) - karras_delta(codes, L, i, i - 1));
    const int dmin = karras_delta(codes, L, i, i - d);
    int lmax = 2;
    while (karras_delta(codes, L, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t > 0; t >>= 1)
      if (karras_delta(codes, L, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = karras_delta(codes, L, i, j);
    int s = 0;
    for (int t = (l + 1) >> 1; t > 0; t = (t == 1 ? 0 : (t + 1) >> 1))
      if (karras_delta(codes, L, i, i + (s + t) * d) > dnode) s += t;
    const int gamma = i + s * d + (d < 0 ? d : 0);
    const int leftIsLeaf = ((i < j ? i : j) == gamma);
    const int rightIsLeaf = ((i > j ? i : j) == gamma + 1);
    nodes[i].leftOffset = (uint32_t)(leftIsLeaf ? (L - 1 + gamma) : gamma);
    nodes[i].escapeIndex = (uint32_t)(rightIsLeaf ? (L - 1 + gamma + 1) : gamma + 1);
  }
}

/* Bottom-up refit of the LR tree.  The reference runs 32 in-place sweeps of
 * kernel1D_RefitPass (core/builders/lbvh.cpp:443-489, :798-802); a node's box is
 * min/max of its two children's boxes and its count is the children's counts
 * plus 2, so the recursive post-order below computes the same values. */
static void refit(ora_node* n, uint32_t* cnt, int L)
{
  if (L < 2) return;
  /* explicit post-order over internal nodes */
  int* stack = (int*)malloc(sizeof(int) * 2 * (size_t)L);
  unsigned char* seen = (unsigned char*)calloc((size_t)L, 1);
  int top = 0;
  stack[top++] = 0;
  while (top > 0)
  {
    const int idx = stack[top - 1];
    const uint32_t l = n[idx].leftOffset, r = n[idx].escapeIndex;
    if (!seen[idx])
    {
      seen[idx] = 1;
      if ((int)r < L - 1) stack[top++] = (int)r;
      if ((int)l < L - 1) stack[top++] = (int)l;
      continue;
    }
    top--;
    for (int c = 0; c < 3; c++)
    {
      n[idx].boxMin[c] = fmin_lm(n[l].boxMin[c], n[r].boxMin[c]);
      n[idx].boxMax[c] = fmax_lm(n[l].boxMax[c], n[r].boxMax[c]);
    }
    cnt[idx] = cnt[l] + cnt[r] + 2;
  }
  free(seen);
  free(stack);
}

/* ---- peach LEFT_OFFSET relayout (core/builders/lbvh.cpp:84-188, 492-729) ---- */

typedef struct { uint32_t x, y; } ora_u2;

static void push_down_escape(ora_u2* le, size_t n, uint32_t left, uint32_t parentEscape) /* lbvh.cpp:141-154 */
{
  /* iterative form of the reference's recursion */
  typedef struct { uint32_t left, esc; } item;
  size_t cap = 64, top = 0;
  item* st = (item*)malloc(sizeof(item) * cap);
  st[top].left = left; st[top].esc = parentEscape; top++;
  while (top > 0)
  {
    const item it = st[--top];
    if (it.left >= n) continue;
    const ora_u2 ln = le[it.left + 0];
    const ora_u2 rn = le[it.left + 1];
    le[it.left + 0].y = it.left + 1;
    le[it.left + 1].y = it.esc;
    if (top + 2 > cap) { cap *= 2; st = (item*)realloc(st, sizeof(item) * cap); }
    /* reference visits left first then right; both writes are independent */
    st[top].left = rn.x; st[top].esc = it.esc; top++;
    st[top].left = ln.x; st[top].esc = it.left + 1; top++;
  }
  free(st);
}

static ora_node dummy_node(void) /* core/builders/cbvh.h:28-36 */
{
  ora_node d;
  memset(&d, 0, sizeof(d));
  d.leftOffset = 0x80000000u;
  d.escapeIndex = 0xFFFFFFFFu;
  return d;
}

static size_t round_up_to(size_t a, size_t b) { while (a % b != 0) a++; return a; }

static void peach_convert(ora_bvh* B)
{
  const size_t nPrims = B->nTris;
  const uint32_t peachSize = (nPrims <= 2048 * 4) ? 256 : 2048; /* PEACHES_MIN / PEACHES_MAX, lbvh.h:25-26 */
  ora_u2 intervals[40];
  int nInt = 0;
  size_t currOffs = 0, currSize = 2, prefixSize = 0;
  if (nPrims == 1)
  {
    intervals[nInt].x = 0; intervals[nInt].y = 2; nInt++;
    currOffs = 2;
  }
  else
  {
    do
    {
      intervals[nInt].x = (uint32_t)currOffs; intervals[nInt].y = (uint32_t)currSize; nInt++;
      currOffs += currSize;
      currSize *= 2;
    } while (currSize < peachSize);
    prefixSize = currSize;
    intervals[nInt].x = (uint32_t)currOffs; intervals[nInt].y = (uint32_t)currSize; nInt++;
    currOffs += currSize;
    currSize *= 2;
    currOffs += currSize;
    currOffs += round_up_to(2 * nPrims - 1, 2);
  }
  const size_t reserved = currOffs;

  /* BuildPeachTree, lbvh.cpp:156-188 */
  ora_u2* le = (ora_u2*)malloc(sizeof(ora_u2) * reserved);
  for (size_t i = 0; i < reserved; i++) { le[i].x = 0xFFFFFFFFu; le[i].y = 0; }
  for (int lv = 0; lv < nInt - 1; lv++)
    for (uint32_t i = intervals[lv].x; i < intervals[lv].x + intervals[lv].y; i++)
    {
      le[i].x = intervals[lv + 1].x + 2 * (i - intervals[lv].x);
      le[i].y = 0;
    }
  push_down_escape(le, reserved, 0, (uint32_t)-2);

  const size_t outSize = reserved + (reserved % 2);
  ora_node* out = (ora_node*)calloc(outSize, sizeof(ora_node));
  ora_u2* addr = (ora_u2*)malloc(sizeof(ora_u2) * reserved);
  for (size_t i = 0; i < reserved; i++) { addr[i].x = 0; addr[i].y = 0; }
  uint32_t* prefix = (uint32_t*)calloc(prefixSize ? prefixSize : 1, sizeof(uint32_t));
  const ora_node* in = B->lr;

  /* kernel1D_PeachConvertInit, lbvh.cpp:492-543 */
  {
    ora_node root = in[0];
    if ((int32_t)root.leftOffset < 0)
    {
      root.escapeIndex = (uint32_t)-2;
      addr[0].x = addr[0].y = 0xFFFFFFFFu;
      addr[1].x = addr[1].y = 0xFFFFFFFFu;
      out[0] = root;
      out[1] = dummy_node();
    }
    else
    {
      const ora_node left = in[root.leftOffset];
      const ora_node right = in[root.escapeIndex];
      addr[0].x = left.leftOffset; addr[0].y = left.escapeIndex;
      addr[1].x = right.leftOffset; addr[1].y = right.escapeIndex;
      ora_node ln = out[0], rn = out[1];
      memcpy(ln.boxMin, left.boxMin, 12); memcpy(ln.boxMax, left.boxMax, 12);
      memcpy(rn.boxMin, right.boxMin, 12); memcpy(rn.boxMax, right.boxMax, 12);
      ln.leftOffset = le[0].x; ln.escapeIndex = le[0].y;
      rn.leftOffset = le[1].x; rn.escapeIndex = le[1].y;
      if ((int32_t)left.leftOffset < 0) { ln.leftOffset = left.leftOffset; addr[0].x = addr[0].y = 0xFFFFFFFFu; }
      if ((int32_t)right.leftOffset < 0) { rn.leftOffset = right.leftOffset; addr[1].x = addr[1].y = 0xFFFFFFFFu; }
      out[0] = ln;
      out[1] = rn;
    }
  }

  /* kernel1D_PeachConvertPass over the perfect levels, lbvh.cpp:545-612 and :806-814 */
  for (int lv = 0; lv < nInt - 1; lv++)
  {
    const uint32_t cs = intervals[lv].x, cn = intervals[lv].y, ns = intervals[lv + 1].x;
    const int last = (lv == nInt - 2);
    for (uint32_t i = 0; i < cn; i++)
    {
      const ora_u2 lr = addr[cs + i];
      int leftIsLeaf = 1, rightIsLeaf = 1;
      for (int side = 0; side < 2; side++)
      {
        const uint32_t src = side ? lr.y : lr.x;
        const size_t dst = ns + 2 * (size_t)i + side;
        if (src == 0xFFFFFFFFu)
        {
          out[dst] = dummy_node();
          addr[dst].x = addr[dst].y = 0xFFFFFFFFu;
        }
        else
        {
          const ora_node ch = in[src];
          const int isLeaf = ((int32_t)ch.leftOffset < 0);
          ora_node nn;
          memcpy(nn.boxMin, ch.boxMin, 12);
          memcpy(nn.boxMax, ch.boxMax, 12);
          nn.leftOffset = isLeaf ? ch.leftOffset : le[dst].x;
          nn.escapeIndex = le[dst].y;
          out[dst] = nn;
          if (isLeaf) { addr[dst].x = addr[dst].y = 0xFFFFFFFFu; }
          else { addr[dst].x = ch.leftOffset; addr[dst].y = ch.escapeIndex; }
          if (side) rightIsLeaf = isLeaf; else leftIsLeaf = isLeaf;
        }
      }
      if (last)
      {
        prefix[2 * i + 0] = leftIsLeaf ? 0 : B->lrCount[lr.x];
        prefix[2 * i + 1] = rightIsLeaf ? 0 : B->lrCount[lr.y];
      }
    }
  }

  /* std::inclusive_scan, lbvh.cpp:816 */
  for (size_t i = 1; i < prefixSize; i++) prefix[i] += prefix[i - 1];

  /* kernel1D_RecursiveConvert over the last perfect level, lbvh.cpp:644-729 and :818-823 */
  if (nInt != 1)
  {
    const uint32_t cs = intervals[nInt - 1].x, cn = intervals[nInt - 1].y;
    for (uint32_t i = 0; i < cn; i++)
    {
      const ora_u2 lr = addr[cs + i];
      uint32_t sub = cs + cn;
      if (i > 0) sub += prefix[i - 1];
      if (lr.x == 0xFFFFFFFFu) continue;
      out[cs + i].leftOffset = sub;
      uint32_t st[32][4];
      int top = 0;
      uint32_t lo = lr.x, ro = lr.y, pe = out[cs + i].escapeIndex;
      while (top >= 0)
      {
        int pop = ((int32_t)lo < 0);
        if ((int32_t)lo > 0)
        {
          const ora_node ln = in[lo];
          const ora_node rn = in[ro];
          const uint32_t cur = sub;
          sub += 2;
          out[cur + 0] = ln;
          out[cur + 1] = rn;
          out[cur + 0].escapeIndex = cur + 1;
          out[cur + 1].escapeIndex = pe;
          pop = ((int32_t)ln.leftOffset < 0) && ((int32_t)rn.leftOffset < 0);
          if ((int32_t)ln.leftOffset > 0 && (int32_t)rn.leftOffset > 0)
          {
            st[top][0] = rn.leftOffset; st[top][1] = rn.escapeIndex; st[top][2] = pe; st[top][3] = cur + 1;
            top++;
          }
          if ((int32_t)ln.leftOffset > 0)
          {
            lo = ln.leftOffset; ro = ln.escapeIndex; pe = cur + 1;
            out[cur + 0].leftOffset = sub;
          }
          else if ((int32_t)rn.leftOffset > 0)
          {
            lo = rn.leftOffset; ro = rn.escapeIndex;
            out[cur + 1].leftOffset = sub;
          }
        }
        if (pop)
        {
          top--;
          const uint32_t* od = st[top > 0 ? top : 0];
          lo = od[0]; ro = od[1]; pe = od[2];
          if ((int32_t)lo > 0 && top >= 0) out[od[3]].leftOffset = sub;
        }
      }
    }
  }

  /* odd size: pad with a dummy node (core/builders/cbvh_hlbvh.cpp:232-236) */
  if (outSize != reserved) out[reserved] = dummy_node();
  /* leaf repack of cbvh.cpp:372-375 maps each leaf (and dummy) word to itself */

  B->nodes = out;
  B->nNodes = (uint32_t)outSize;
  free(prefix);
  free(addr);
  free(le);
}

/* Whole build: scene box, Morton codes, stable sort, run compaction, leaves,
 * Karras hierarchy, refit, peach relayout; then the per-geometry arrays that
 * BVH2CommonRT::AddGeom_Triangles3f keeps (core/BVH2CommonRT_host.cpp:45-98). */
ora_bvh* ora_build(const float* v4, uint32_t nV, const uint32_t* idx, uint32_t nIdx)
{
  ora_bvh* B = (ora_bvh*)calloc(1, sizeof(ora_bvh));
  const uint32_t N = nIdx / 3;
  B->nTris = N;
  B->nVerts = nV;
  B->verts = (float*)malloc(sizeof(float) * 4 * (size_t)(nV ? nV : 1));
  for (uint32_t i = 0; i < nV; i++)
  {
    B->verts[4 * i + 0] = v4[4 * i + 0];
    B->verts[4 * i + 1] = v4[4 * i + 1];
    B->verts[4 * i + 2] = v4[4 * i + 2];
    B->verts[4 * i + 3] = 1.0f;
  }
  if (N == 0) return B;

  aabb_from_vertices(B->verts, nV, B->bmin, B->bmax);
  zindex_scale(B->bmin, B->bmax, B->scale);
  B->pairsUnsorted = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)N);
  morton_codes(B->verts, idx, N, B->bmin, B->scale, B->pairsUnsorted);
  B->pairsSorted = (uint32_t*)malloc(sizeof(uint32_t) * 2 * (size_t)N);
  memcpy(B->pairsSorted, B->pairsUnsorted, sizeof(uint32_t) * 2 * (size_t)N);
  sort_pairs_stable(B->pairsSorted, N);

  /* kernel1D_AppendInit + exclusive_scan + AppendComplete, lbvh.cpp:289-319,762-767 */
  uint32_t L = 0;
  for (uint32_t i = 0; i < N; i++)
    if (i == 0 || B->pairsSorted[2 * (i - 1)] != B->pairsSorted[2 * i]) L++;
  B->nLeaves = L;
  B->compressed = (uint32_t*)malloc(sizeof(uint32_t) * L);
  B->runStarts = (uint32_t*)malloc(sizeof(uint32_t) * L);
  for (uint32_t i = 0, w = 0; i < N; i++)
    if (i == 0 || B->pairsSorted[2 * (i - 1)] != B->pairsSorted[2 * i])
    {
      B->compressed[w] = B->pairsSorted[2 * i];
      B->runStarts[w] = i;
      w++;
    }

  /* kernel1D_MakeLeavesFromTriangles, lbvh.cpp:350-384: leaf i sits at node L-1+i */
  const uint32_t nLR = 2 * L - 1;
  B->lr = (ora_node*)calloc(nLR, sizeof(ora_node));
  B->lrCount = (uint32_t*)calloc(nLR, sizeof(uint32_t));
  B->leafIndices = (uint32_t*)malloc(sizeof(uint32_t) * N);
  for (uint32_t i = 0; i < L; i++)
  {
    const uint32_t start = B->runStarts[i];
    const uint32_t count = (i + 1 < L) ? B->runStarts[i + 1] - start : N - start;
    if (count > 127) B->status = 1; /* the reference's 7-bit count field overflows here */
    float mn[3] = {1e10f, 1e10f, 1e10f}, mx[3] = {-1e10f, -1e10f, -1e10f};
    for (uint32_t j = start; j < start + count; j++)
    {
      const uint32_t tri = B->pairsSorted[2 * j + 1];
      B->leafIndices[j] = tri;
      const float* a = B->verts + 4 * (size_t)idx[3 * tri + 0];
      const float* b = B->verts + 4 * (size_t)idx[3 * tri + 1];
      const float* c = B->verts + 4 * (size_t)idx[3 * tri + 2];
      for (int k = 0; k < 3; k++)
      {
        mn[k] = fmin_lm(mn[k], fmin_lm(a[k], fmin_lm(b[k], c[k])));
        mx[k] = fmax_lm(mx[k], fmax_lm(a[k], fmax_lm(b[k], c[k])));
      }
    }
    ora_node* nd = &B->lr[L - 1 + i];
    memcpy(nd->boxMin, mn, 12);
    memcpy(nd->boxMax, mx, 12);
    nd->leftOffset = pack_offset_and_size(start, count);
    nd->escapeIndex = 0xFFFFFFFFu;
  }
  karras12(B->compressed, (int)L, B->lr);
  refit(B->lr, B->lrCount, (int)L);
  peach_convert(B);

  /* AppendTreeData, core/BVH2CommonRT_host.cpp:45-64 */
  B->indicesSorted = (uint32_t*)malloc(sizeof(uint32_t) * 3 * (size_t)N);
  for (uint32_t i = 0; i < N; i++)
  {
    const uint32_t tri = B->leafIndices[i];
    B->indicesSorted[3 * i + 0] = idx[3 * tri + 0];
    B->indicesSorted[3 * i + 1] = idx[3 * tri + 1];
    B->indicesSorted[3 * i + 2] = idx[3 * tri + 2];
  }
  return B;
}

void ora_free(ora_bvh* B)
{
  if (!B) return;
  free(B->pairsUnsorted); free(B->pairsSorted); free(B->compressed); free(B->runStarts);
  free(B->lr); free(B->lrCount); free(B->leafIndices); free(B->nodes); free(B->indicesSorted); free(B->verts);
  free(B);
}

/* accessors for ctypes */
uint32_t ora_num_tris(const ora_bvh* B) { return B->nTris; }
uint32_t ora_num_leaves(const ora_bvh* B) { return B->nLeaves; }
uint32_t ora_num_nodes(const ora_bvh* B) { return B->nNodes; }
int ora_status(const ora_bvh* B) { return B->status; }
void ora_get_box(const ora_bvh* B, float* out12)
{
  memcpy(out12, B->bmin, 16); memcpy(out12 + 4, B->bmax, 16); memcpy(out12 + 8, B->scale, 16);
}
void ora_copy_u32(const ora_bvh* B, int which, uint32_t* out)
{
  const uint32_t N = B->nTris, L = B->nLeaves;
  switch (which)
  {
    case 0: memcpy(out, B->pairsUnsorted, 8 * (size_t)N); break;
    case 1: memcpy(out, B->pairsSorted, 8 * (size_t)N); break;
    case 2: memcpy(out, B->compressed, 4 * (size_t)L); break;
    case 3: memcpy(out, B->runStarts, 4 * (size_t)L); break;
    case 4: memcpy(out, B->lr, sizeof(ora_node) * (size_t)(2 * L - 1)); break;
    case 5: memcpy(out, B->lrCount, 4 * (size_t)(2 * L - 1)); break;
    case 6: memcpy(out, B->leafIndices, 4 * (size_t)N); break;
    case 7: memcpy(out, B->nodes, sizeof(ora_node) * (size_t)B->nNodes); break;
    case 8: memcpy(out, B->indicesSorted, 12 * (size_t)N); break;
    default: break;
  }
}

/* ------------------------------------------------------------------ traversal */

/* SafeInverse, core/raytrace_common.h:57-65 */
static inline float safe_inv(float d)
{
  const float ooeps = 1.0e-36f;
  return 1.0f / (fabsf(d) > ooeps ? d : copysignf(ooeps, d));
}

/* RayBoxIntersection2, core/raytrace_common.h:67-80 */
static inline void ray_box(const float o[3], const float inv[3], const float* bmin, const float* bmax, float* tn, float* tf)
{
  const float lo = inv[0] * (bmin[0] - o[0]);
  const float hi = inv[0] * (bmax[0] - o[0]);
  const float lo1 = inv[1] * (bmin[1] - o[1]);
  const float hi1 = inv[1] * (bmax[1] - o[1]);
  const float lo2 = inv[2] * (bmin[2] - o[2]);
  const float hi2 = inv[2] * (bmax[2] - o[2]);
  const float tmin = fmax_std(fmin_std(lo, hi), fmin_std(lo1, hi1));
  const float tmax = fmin_std(fmax_std(lo, hi), fmax_std(lo1, hi1));
  *tn = fmax_std(tmin, fmin_std(lo2, hi2));
  *tf = fmin_std(tmax, fmax_std(lo2, hi2));
}

/* IntersectAllPrimitivesInLeaf, core/BVH2CommonRT.cpp:9-47 (single geometry,
 * offsets 0).  Returns 1 if a triangle was accepted. */
static inline int leaf_test(const ora_bvh* B, const float o[3], const float d[3], float tNear, uint32_t start,
                            uint32_t count, ora_hit* hit)
{
  int found = 0;
  for (uint32_t tri = start; tri < start + count; tri++)
  {
    const float* A = B->verts + 4 * (size_t)B->indicesSorted[3 * tri + 0];
    const float* Bv = B->verts + 4 * (size_t)B->indicesSorted[3 * tri + 1];
    const float* C = B->verts + 4 * (size_t)B->indicesSorted[3 * tri + 2];
    const float e1[3] = {Bv[0] - A[0], Bv[1] - A[1], Bv[2] - A[2]};
    const float e2[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
    const float pv[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
    const float tv[3] = {o[0] - A[0], o[1] - A[1], o[2] - A[2]};
    const float qv[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
    const float invDet = 1.0f / (e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2]);
    const float v = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) * invDet;
    const float u = (qv[0] * d[0] + qv[1] * d[1] + qv[2] * d[2]) * invDet;
    const float t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * invDet;
    if (v >= -1e-6f && u >= -1e-6f && (u + v <= 1.0f + 1e-6f) && t > tNear && t < hit->t)
    {
      hit->t = t;
      hit->primId = tri;
      hit->instId = 0;
      hit->geomId = 0;
      hit->coords[0] = u;
      hit->coords[1] = v;
      found = 1;
    }
  }
  return found;
}

/* BVH2TraverseC32, core/BVH2CommonRT.cpp:49-141, on the peach node array.
 * anyHit != 0 stops at the first accepted triangle, as the reference's siblings
 * do for RayQuery_AnyHit (core/BVH2CommonRTStacklessLBVH.cpp:65,161-165).
 * counters (optional): [0] node pairs loaded, [1] triangles tested. */
static void traverse(const ora_bvh* B, const float* ray8, int anyHit, ora_hit* hit, uint64_t* counters)
{
  const float o[3] = {ray8[0], ray8[1], ray8[2]};
  const float tNear = ray8[3];
  const float d[3] = {ray8[4], ray8[5], ray8[6]};
  hit->t = ray8[7];
  hit->primId = hit->instId = hit->geomId = 0xFFFFFFFFu;
  hit->coords[0] = hit->coords[1] = hit->coords[2] = hit->coords[3] = 0.0f;
  if (B->nTris == 0) return;
  const float inv[3] = {safe_inv(d[0]), safe_inv(d[1]), safe_inv(d[2])};
  uint32_t stack[ORA_STACK_SIZE];
  stack[0] = 0;
  int top = 0;
  uint32_t off = 0;
  while (top >= 0)
  {
    int pop = 0;
    if ((off & ORA_LEAF_BIT) == 0)
    {
      const ora_node* n0 = &B->nodes[off + 0];
      const ora_node* n1 = &B->nodes[off + 1];
      float t0n, t0f, t1n, t1f;
      ray_box(o, inv, n0->boxMin, n0->boxMax, &t0n, &t0f);
      ray_box(o, inv, n1->boxMin, n1->boxMax, &t1n, &t1f);
      if (counters) counters[0]++;
      const int h0 = (t0n <= t0f) && (t0f >= tNear) && (t0n <= hit->t);
      const int h1 = (t1n <= t1f) && (t1f >= tNear) && (t1n <= hit->t);
      pop = (!h0 && !h1);
      off = h0 ? n0->leftOffset : n1->leftOffset;
      if (h0 && h1)
      {
        off = (t0n <= t1n) ? n0->leftOffset : n1->leftOffset;
        stack[top] = (t0n <= t1n) ? n1->leftOffset : n0->leftOffset;
        top++;
      }
    }
    else if (off != 0xFFFFFFFFu)
    {
      const uint32_t start = off & ORA_START_MASK;
      const uint32_t count = (off & ORA_SIZE_MASK) >> 24;
      if (counters) counters[1] += count;
      const int found = leaf_test(B, o, d, tNear, start, count, hit);
      if (anyHit && found) return;
      pop = 1;
    }
    if (pop)
    {
      top--;
      off = stack[top > 0 ? top : 0];
    }
  }
}

/* Batch traversal over interleaved rays {posAndNear, dirAndFar} (8 floats per
 * ray).  mode 0: nearest hit into hits[]; mode 1: any hit into any[] (0/1).
 * counters (optional, 2 entries) sum node pairs and triangle tests.  Returns
 * the number of threads used. */
int ora_trace(const ora_bvh* B, const float* rays, uint64_t n, int mode, ora_hit* hits, uint8_t* any, int threads,
              uint64_t* counters)
{
  int used = 1;
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
  used = threads;
#else
  (void)threads;
#endif
  uint64_t c0 = 0, c1 = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(used) reduction(+ : c0, c1)
#endif
  for (int64_t i = 0; i < (int64_t)n; i++)
  {
    ora_hit h;
    uint64_t cnt[2] = {0, 0};
    traverse(B, rays + 8 * (size_t)i, mode == 1, &h, counters ? cnt : NULL);
    c0 += cnt[0];
    c1 += cnt[1];
    if (mode == 1) any[i] = (h.geomId != 0xFFFFFFFFu) ? 1 : 0;
    else hits[i] = h;
  }
  if (counters) { counters[0] = c0; counters[1] = c1; }
  return used;
}

/* ---------------------------------------------------------------- ray set-up
 * Eye rays of HeavyRT's renderers: RTAO::kernel_InitEyeRay
 * (examples/02_rtao/rtao.cpp:133-144; the same body in
 * examples/01_eye_rays/eye_ray.cpp:26-47) with EyeRayDirNormalized and
 * transform_ray3f (examples/render_common.h:6-12,20-36), one ray per pixel
 * centre in row-major order.  Matrices are column-major; mat x vec sums
 * ((m0*x + m1*y) + m2*z) + m3*w per row, normalize(v) = v * (1/sqrt(dot(v,v)))
 * with dot = (x*x + y*y) + z*z, as the LiteMath stand-in evaluates them. */
static void ora_mat_vec(const float* m, const float v[4], float o[4])
{
  for (int r = 0; r < 4; r++) o[r] = ((m[r] * v[0] + m[4 + r] * v[1]) + m[8 + r] * v[2]) + m[12 + r] * v[3];
}

static void ora_normalize3(float v[3])
{
  const float inv = 1.0f / sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
  v[0] = v[0] * inv;
  v[1] = v[1] * inv;
  v[2] = v[2] * inv;
}

void ora_eye_rays(const float* projInv, const float* worldViewInv, uint32_t width, uint32_t height, float tNear,
                  float tFar, float* rays)
{
  for (uint32_t y = 0; y < height; y++)
    for (uint32_t x = 0; x < width; x++)
    {
      const float fx = ((float)x + 0.5f) / (float)width, fy = ((float)y + 0.5f) / (float)height;
      const float pos[4] = {2.0f * fx - 1.0f, -2.0f * fy + 1.0f, 0.0f, 1.0f};
      float p[4];
      ora_mat_vec(projInv, pos, p);
      const float w = p[3];
      float d[3] = {p[0] / w, p[1] / w, p[2] / w};
      ora_normalize3(d);
      const float o0[4] = {0.0f, 0.0f, 0.0f, 1.0f};
      const float o1[4] = {0.0f + 100.0f * d[0], 0.0f + 100.0f * d[1], 0.0f + 100.0f * d[2], 1.0f};
      float a[4], b[4];
      ora_mat_vec(worldViewInv, o0, a);
      ora_mat_vec(worldViewInv, o1, b);
      float dir[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
      ora_normalize3(dir);
      float* r = rays + 8 * ((size_t)y * width + x);
      r[0] = a[0]; r[1] = a[1]; r[2] = a[2]; r[3] = tNear;
      r[4] = dir[0]; r[5] = dir[1]; r[6] = dir[2]; r[7] = tFar;
    }
}
