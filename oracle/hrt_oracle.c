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

/* ZIndexMultCoeff on the biased box, core/builders/lbvh.cpp:41-51 and :263.
 * cubic != 0 restates the engine's HRT_MORTON_CUBIC frame (no reference
 * counterpart): x, y and z take the scale of the longest biased extent. */
static void zindex_scale(const float bmin[4], const float bmax[4], float scale[4], int cubic)
{
  float ext[4];
  for (int c = 0; c < 4; c++)
  {
    const float lo = bmin[c] - 1e-4f;
    const float hi = bmax[c] + 1e-4f;
    ext[c] = hi - lo;
  }
  const float emax = fmax_lm(ext[0], fmax_lm(ext[1], ext[2]));
  for (int c = 0; c < 4; c++)
  {
    const float e = (cubic && c < 3) ? emax : ext[c];
    float inv = 1.0f / e;
    if (c < 3 && fabsf(e) < 1e-20f) inv = 0.0f;
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
  int       triTest;       /* 0 the reference's Moller-Trumbore, 1 watertight */
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
ora_bvh* ora_build_frame(const float* v4, uint32_t nV, const uint32_t* idx, uint32_t nIdx, int cubic);

ora_bvh* ora_build(const float* v4, uint32_t nV, const uint32_t* idx, uint32_t nIdx)
{
  return ora_build_frame(v4, nV, idx, nIdx, 0);
}

/* The same build on the engine's cubic Morton grid when cubic != 0. */
ora_bvh* ora_build_frame(const float* v4, uint32_t nV, const uint32_t* idx, uint32_t nIdx, int cubic)
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
  zindex_scale(B->bmin, B->bmax, B->scale, cubic);
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
/* 0: the reference's Moller-Trumbore test (default), 1: the watertight test. */
void ora_set_triangle_test(ora_bvh* B, int test) { B->triTest = test; }
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

/* Watertight ray-triangle test of Woop, Benthin & Wald ("Watertight
 * Ray/Triangle Intersection", JCGT 2(1), 2013), restated for the engine's
 * HRT_TRI_WATERTIGHT mode (not a reference function: HeavyRT has only the
 * Moller-Trumbore test above).  The ray's dominant axis becomes z (kx, ky
 * swapped when that component is negative, keeping the winding), vertices are
 * translated to the ray origin and sheared, and the signs of the three edge
 * functions U, V, W at the origin decide the hit, both windings accepted.  The
 * paper's double-precision re-evaluation of a zero edge function is replaced
 * by Kahan's difference of products (one product's rounding error restored by
 * a fused multiply-add), whose relative error is below 2 ulp, so every sign is
 * exact in binary32.  t = T / det as T * (1 / det); coords = (W, V) / det, the
 * weights of C and B, the fields the Moller-Trumbore test fills.  fmaf is the
 * correctly rounded fused multiply-add on every platform. */
static inline float ora_pick3(const float v[3], int k) { return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]); }

static inline float ora_diff_of_products(float a, float b, float c, float d)
{
  const float w = c * d;
  const float e = fmaf(-c, d, w);
  const float f = fmaf(a, b, -w);
  return f + e;
}

static inline int leaf_test_wt(const ora_bvh* B, const float o[3], const float d[3], float tNear, uint32_t start,
                               uint32_t count, ora_hit* hit)
{
  const float ad[3] = {fabsf(d[0]), fabsf(d[1]), fabsf(d[2])};
  const int kz = (ad[0] >= ad[1] && ad[0] >= ad[2]) ? 0 : (ad[1] >= ad[2] ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  const float dz = ora_pick3(d, kz);
  if (dz < 0.0f)
  {
    const int t = kx;
    kx = ky;
    ky = t;
  }
  const float sx = ora_pick3(d, kx) / dz, sy = ora_pick3(d, ky) / dz, sz = 1.0f / dz;
  int found = 0;
  for (uint32_t tri = start; tri < start + count; tri++)
  {
    const float* V0 = B->verts + 4 * (size_t)B->indicesSorted[3 * tri + 0];
    const float* V1 = B->verts + 4 * (size_t)B->indicesSorted[3 * tri + 1];
    const float* V2 = B->verts + 4 * (size_t)B->indicesSorted[3 * tri + 2];
    const float a[3] = {V0[0] - o[0], V0[1] - o[1], V0[2] - o[2]};
    const float b[3] = {V1[0] - o[0], V1[1] - o[1], V1[2] - o[2]};
    const float c[3] = {V2[0] - o[0], V2[1] - o[1], V2[2] - o[2]};
    const float az = ora_pick3(a, kz), bz = ora_pick3(b, kz), cz = ora_pick3(c, kz);
    const float ax = ora_pick3(a, kx) - sx * az, ay = ora_pick3(a, ky) - sy * az;
    const float bx = ora_pick3(b, kx) - sx * bz, by = ora_pick3(b, ky) - sy * bz;
    const float cx = ora_pick3(c, kx) - sx * cz, cy = ora_pick3(c, ky) - sy * cz;
    const float U = ora_diff_of_products(cx, by, cy, bx);
    const float V = ora_diff_of_products(ax, cy, ay, cx);
    const float W = ora_diff_of_products(bx, ay, by, ax);
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) continue;
    const float det = (U + V) + W;
    if (det == 0.0f) continue;
    const float T = (U * (sz * az) + V * (sz * bz)) + W * (sz * cz);
    const float inv = 1.0f / det;
    const float t = T * inv;
    if (t > tNear && t < hit->t)
    {
      hit->t = t;
      hit->primId = tri;
      hit->instId = 0;
      hit->geomId = 0;
      hit->coords[0] = W * inv;
      hit->coords[1] = V * inv;
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
      const int found = B->triTest ? leaf_test_wt(B, o, d, tNear, start, count, hit)
                                   : leaf_test(B, o, d, tNear, start, count, hit);
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

/* ---------------------------------------------------------------- renderer frames
 * The frame kernels of HeavyRT's two example renderers, restated per ray /
 * per pixel as the reference evaluates them under the LiteMath stand-in
 * (float operations left to right; the unqualified sin, cos, pow and sqrt
 * that examples/render_common.h calls on float arguments resolve to the double
 * functions of <math.h>, std::sqrt / std::pow / std::abs to the float ones). */

/* EyeRayCaster's palette (examples/01_eye_rays/eye_ray.h:105-113). */
static const uint32_t ora_palette[20] = {
    0xffe6194bu, 0xff3cb44bu, 0xffffe119u, 0xff0082c8u, 0xfff58231u, 0xff911eb4u, 0xff46f0f0u,
    0xfff032e6u, 0xffd2f53cu, 0xfffabebeu, 0xff008080u, 0xffe6beffu, 0xffaa6e28u, 0xfffffac8u,
    0xff800000u, 0xffaaffc3u, 0xff808000u, 0xffffd8b1u, 0xff000080u, 0xff808080u};

/* kernel_PackXY with SuperBlockIndex2DOpt (examples/01_eye_rays/eye_ray.cpp:106-134):
 * packed[offset(x, y)] = y << 16 | x, 4x4 blocks inside 2x2 super-blocks.
 * Offsets at or past width*height are skipped (the reference writes past its
 * array there: widths or heights that are not multiples of 8). */
void ora_pack_xy(uint32_t width, uint32_t height, uint32_t* packed)
{
  const uint32_t n = width * height;
  for (uint32_t y = 0; y < height; y++)
    for (uint32_t x = 0; x < width; x++)
    {
      const uint32_t local = (y & 3u) * 4u + (x & 3u);
      const uint32_t bx = x >> 2, by = y >> 2;
      const uint32_t localH = (by & 1u) * 2u + (bx & 1u);
      const uint32_t wH = (width >> 2) >> 1;
      const uint32_t off = ((bx >> 1) + (by >> 1) * wH) * 64u + localH * 16u + local;
      if (off < n) packed[off] = ((y << 16) & 0xFFFF0000u) | (x & 0x0000FFFFu);
    }
}

/* kernel_RayTrace (examples/01_eye_rays/eye_ray.cpp:49-74), one colour per hit. */
void ora_eye_colors(const ora_hit* hits, uint64_t n, uint32_t* colors)
{
  for (uint64_t i = 0; i < n; i++)
    colors[i] = hits[i].primId == 0xFFFFFFFFu ? 0u : ora_palette[hits[i].primId % 20u];
}

/* Niederreiter base-2 direction numbers for 4 dimensions, as
 * initQuasirandomGenerator computes them (core/common/qmc_sobol_niederreiter.cpp:
 * GeneratePolynomials :13-67, GenerateCJ :81-174, table :179-186; Bratley, Fox and
 * Niederreiter, ACM TOMACS 2(3), 1992).  Dimension d uses the d-th irreducible
 * polynomial over GF(2) in numeric order (x, x+1, x^2+x+1, x^3+x+1).  Output bit r
 * (r = 0 most significant) of row i is v[i + r mod e] of the linear recurrence
 * with characteristic polynomial P^(r div e + 1), started from r div e * e zeros
 * followed by ones up to that polynomial's degree.  table[d*31 + i] keeps bits
 * 62..32 of the reference's 63-bit words. */
static int gf2_deg(uint32_t p)
{
  int d = 31;
  while (d > 0 && !((p >> d) & 1u)) d--;
  return d;
}

static uint32_t gf2_rem(uint32_t a, uint32_t b)
{
  const int db = gf2_deg(b);
  while (a != 0 && gf2_deg(a) >= db) a ^= b << (gf2_deg(a) - db);
  return a;
}

void ora_qmc_table(uint32_t* table)
{
  uint32_t polys[4] = {2u, 0u, 0u, 0u};
  for (int n = 1; n < 4; n++)
    for (uint32_t p = polys[n - 1] + 1u;; p++)
    {
      int irreducible = 1;
      for (int k = 0; k < n && irreducible; k++) irreducible = gf2_rem(p, polys[k]) != 0u;
      if (irreducible) { polys[n] = p; break; }
    }
  for (int d = 0; d < 4; d++)
  {
    const uint32_t P = polys[d];
    const int e = gf2_deg(P);
    uint8_t pc[33];                      /* P's coefficients, pc[k] = coefficient of x^(e-k) */
    for (int k = 0; k <= e; k++) pc[k] = (uint8_t)((P >> (e - k)) & 1u);
    uint8_t b[64] = {1}, t[64];          /* b = P^q, b[k] = coefficient of x^(deg-k) */
    int m = 0;
    for (int i = 0; i < 31; i++) table[d * 31 + i] = 0u;
    for (int r = 0; r < 31; r++)
    {
      const int u = r % e;
      if (u == 0)
      {
        const int m1 = m;
        memcpy(t, b, sizeof(b));
        m = m1 + e;
        for (int i = 0; i <= m; i++)
        {
          uint8_t c = 0;
          for (int k = 0; k <= e; k++)
            if (i - k >= 0 && i - k <= m1) c ^= (uint8_t)(pc[k] & t[i - k]);
          b[i] = c;
        }
      }
      uint8_t v[96];
      const int m1 = m - e;
      const int len = 31 + e;
      for (int i = 0; i < len; i++)
      {
        if (i < m1) v[i] = 0;
        else if (i < m) v[i] = 1;
        else
        {
          uint8_t s = 0;
          for (int k = 1; k <= m; k++) s ^= (uint8_t)(v[i - k] & b[k]);
          v[i] = s;
        }
      }
      for (int i = 0; i < 31; i++) table[d * 31 + i] |= (uint32_t)v[i + u] << (30 - r);
    }
  }
}

/* rndQmcSobolN (core/common/qmc_sobol_niederreiter.h:11-20). */
static float ora_qmc(const uint32_t* table, uint32_t pos, int dim)
{
  uint32_t result = 0;
  for (int bit = 0; bit < 31; bit++, pos >>= 1)
    if (pos & 1u) result ^= table[bit + dim * 31];
  return (float)(result + 1u) * (1.0f / (float)0x80000001u);
}

/* RTAO::InitQMCTable (examples/02_rtao/rtao_host.cpp:383-414): 128x128 texels of
 * raysPerPixel (r1, r2) pairs; unfilled entries stay (0, 0). */
void ora_rtao_tile(uint32_t raysPerPixel, float* tile)
{
  uint32_t table[4 * 31];
  ora_qmc_table(table);
  const size_t n = (size_t)128 * 128 * raysPerPixel;
  uint32_t* filled = (uint32_t*)calloc(128 * 128, sizeof(uint32_t));
  memset(tile, 0, sizeof(float) * 2 * n);
  for (size_t i = 0; i < n; i++)
  {
    const float x = ora_qmc(table, (uint32_t)i, 0), y = ora_qmc(table, (uint32_t)i, 1);
    const float z = ora_qmc(table, (uint32_t)i, 2), w = ora_qmc(table, (uint32_t)i, 3);
    int ix = (int)(x * 128.0f), iy = (int)(y * 128.0f);
    if (ix >= 128) ix = 127;
    if (iy >= 128) iy = 127;
    const uint32_t cell = (uint32_t)iy * 128u + (uint32_t)ix;
    if (filled[cell] < raysPerPixel)
    {
      float* o = tile + 2 * ((size_t)cell * raysPerPixel + filled[cell]);
      o[0] = z;
      o[1] = w;
      filled[cell]++;
    }
  }
  free(filled);
}

/* LiteMath normalize under the stand-in: v * (1 / std::sqrt(dot(v, v))). */
static void ora_norm3(float v[3])
{
  const float l = sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
  const float inv = 1.0f / l;
  v[0] = v[0] * inv;
  v[1] = v[1] * inv;
  v[2] = v[2] * inv;
}

/* mymul3x3 (examples/render_common.h:14-17): the full column sum with w = 0. */
static void ora_mul3x3(const float* m, const float v[3], float o[3])
{
  for (int r = 0; r < 3; r++) o[r] = ((m[r] * v[0] + m[4 + r] * v[1]) + m[8 + r] * v[2]) + m[12 + r] * 0.0f;
}

static inline float ora_dot3(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

/* C++ float -> int conversion, with the NaN case (undefined in C++) mapped to 0. */
static inline int ora_f2i(float f) { return f != f ? 0 : (int)f; }

/* encodeNormal / decodeNormal (examples/render_common.h:114-137). */
static uint32_t ora_encode_normal(const float n[3])
{
  const int x = ora_f2i(n[0] * 32767.0f);
  const int y = ora_f2i(n[1] * 32767.0f);
  const uint32_t sign = (n[2] >= 0) ? 0u : 1u;
  const uint32_t sx = ((uint32_t)(x & 0xfffe) | sign);
  const uint32_t sy = ((uint32_t)(y & 0xffff) << 16);
  return sx | sy;
}

static void ora_decode_normal(uint32_t a, float n[3])
{
  const uint32_t ex = a & 0x0000FFFFu, ey = (a & 0xFFFF0000u) >> 16;
  const float sign = (ex & 1u) != 0 ? -1.0f : 1.0f;
  const float k = 1.0f / 32767.0f;
  n[0] = (float)(int16_t)(uint16_t)(ex & 0xfffeu) * k;
  n[1] = (float)(int16_t)(uint16_t)(ey & 0xffffu) * k;
  n[2] = sign * sqrtf(fmax_std((1.0f - n[0] * n[0]) - n[1] * n[1], 0.0f));
}

/* RTAO::kernel_TraceEyeRay2 after its query (examples/02_rtao/rtao.cpp:81-131):
 * the hit position pulled back by 0.9999995 t and the shading normal (vertex
 * normals interpolated, both normals through the instance's normal matrix,
 * flipped towards the triangle's side facing the ray) packed into w.  A hit's
 * triangle is read from the geometry's index buffer in sorted order at the
 * hit's primId (the sorted position), i.e. the triangle that was hit.
 * sortedIdx[g], verts[g] (float4), normals[g] (float4) per geometry;
 * normMatrices: 16 floats per instance, column-major. */
void ora_rtao_positions(const float* eyeRays, const ora_hit* hits, uint64_t n, const uint32_t* const* sortedIdx,
                        const float* const* verts, const float* const* normals, const float* normMatrices,
                        float* positions)
{
  for (uint64_t i = 0; i < n; i++)
  {
    const ora_hit h = hits[i];
    float* out = positions + 4 * i;
    if (h.geomId == 0xFFFFFFFFu)
    {
      const float up[3] = {0.0f, 1.0f, 0.0f};
      const uint32_t e = ora_encode_normal(up);
      out[0] = 0.0f; out[1] = 10000000.0f; out[2] = 0.0f;
      memcpy(out + 3, &e, 4);
      continue;
    }
    const float* o = eyeRays + 8 * i;
    const float* d = o + 4;
    const float u = h.coords[0], v = h.coords[1];
    const float s = 0.9999995f * h.t;
    const float p[3] = {o[0] + s * d[0], o[1] + s * d[1], o[2] + s * d[2]};
    const uint32_t* tri = sortedIdx[h.geomId] + 3 * (size_t)h.primId;
    const float* A = verts[h.geomId] + 4 * (size_t)tri[0];
    const float* B = verts[h.geomId] + 4 * (size_t)tri[1];
    const float* Cv = verts[h.geomId] + 4 * (size_t)tri[2];
    const float e1[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
    const float e2[3] = {Cv[0] - A[0], Cv[1] - A[1], Cv[2] - A[2]};
    const float tn0[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const float* nA = normals[h.geomId] + 4 * (size_t)tri[0];
    const float* nB = normals[h.geomId] + 4 * (size_t)tri[1];
    const float* nC = normals[h.geomId] + 4 * (size_t)tri[2];
    const float w0 = (1.0f - u) - v;
    float hn0[3];
    for (int k = 0; k < 3; k++) hn0[k] = (w0 * nA[k] + v * nB[k]) + u * nC[k];
    const float* M = normMatrices + 16 * (size_t)h.instId;
    float hn[3], tn[3];
    ora_mul3x3(M, hn0, hn);
    ora_norm3(hn);
    ora_mul3x3(M, tn0, tn);
    ora_norm3(tn);
    if (ora_dot3(tn, hn) < 0.0f)
      for (int k = 0; k < 3; k++) hn[k] = hn[k] * -1.0f;
    const float dotp = ora_dot3(d, tn);
    const float flip = (dotp > 1e-5f) ? -1.0f : 1.0f;
    const float fn[3] = {hn[0] * flip, hn[1] * flip, hn[2] * flip};
    const uint32_t e = ora_encode_normal(fn);
    out[0] = p[0]; out[1] = p[1]; out[2] = p[2];
    memcpy(out + 3, &e, 4);
  }
}

/* RTAO::kernel_InitAORay (examples/02_rtao/rtao.cpp:147-165) with
 * MapSampleToCosineDistribution (power 1), CoordinateSystem and OffsRayPos
 * (examples/render_common.h:38-112), for every pixel (row-major) and sample z:
 * aoRays[(pix*R + z)*8 ..] = {pos, 0, dir, aoMaxRadius}; pixels without a hit
 * (positions y >= 1e7) get no rays (left as they are). */
void ora_rtao_ao_rays(const float* positions, uint32_t width, uint32_t height, uint32_t R, const float* tile,
                      float aoMaxRadius, float* aoRays)
{
  const float twoPi = 6.28318530717958647692f;
  for (uint32_t y = 0; y < height; y++)
    for (uint32_t x = 0; x < width; x++)
    {
      const size_t pix = (size_t)y * width + x;
      const float* pos = positions + 4 * pix;
      if (pos[1] >= 10000000.0f) continue;
      uint32_t enc;
      memcpy(&enc, pos + 3, 4);
      float nrm[3];
      ora_decode_normal(enc, nrm);
      /* CoordinateSystem(normal): nx, then nz = cross(normal, nx) */
      float nx[3], invLen;
      if (fabsf(nrm[0]) > fabsf(nrm[1]))
      {
        invLen = 1.0f / sqrtf(nrm[0] * nrm[0] + nrm[2] * nrm[2]);
        nx[0] = (-1.0f * nrm[2]) * invLen; nx[1] = 0.0f; nx[2] = nrm[0] * invLen;
      }
      else
      {
        invLen = (float)(1.0f / sqrt((double)(nrm[1] * nrm[1] + nrm[2] * nrm[2])));
        nx[0] = 0.0f; nx[1] = nrm[2] * invLen; nx[2] = (-1.0f * nrm[1]) * invLen;
      }
      const float v3[3] = {nrm[1] * nx[2] - nrm[2] * nx[1], nrm[2] * nx[0] - nrm[0] * nx[2], nrm[0] * nx[1] - nrm[1] * nx[0]};
      const float* ny = v3;   /* after the swap: ny = cross, nz = the normal */
      const float* nz = nrm;
      const float invSign = ora_dot3(nrm, nrm) > 0.0f ? 1.0f : -1.0f;
      const float eps = fmax_std(fmax_std(fabsf(pos[0]), fmax_std(fabsf(pos[1]), fabsf(pos[2]))), 2.0f * 2e-5f) * 2e-5f;
      for (uint32_t z = 0; z < R; z++)
      {
        const float* uv = tile + 2 * (((size_t)(y % 128u) * 128u + (x % 128u)) * R + z);
        const float r1 = uv[0], r2 = uv[1];
        const float phi = twoPi * r1;
        const float sinPhi = (float)sin((double)phi);
        const float cosPhi = (float)cos((double)phi);
        const float cosTheta = (float)pow((double)(1.0f - r2), (double)(1.0f / (1.0f + 1.0f)));
        const float sinTheta = (float)sqrt((double)(1.0f - cosTheta * cosTheta));
        const float dev[3] = {sinTheta * cosPhi, sinTheta * sinPhi, cosTheta};
        float res[3];
        for (int k = 0; k < 3; k++) res[k] = (nx[k] * dev[0] + ny[k] * dev[1]) + nz[k] * dev[2];
        if (invSign * ora_dot3(res, nrm) < 0.0f)
          for (int k = 0; k < 3; k++) res[k] = ((-1.0f * nx[k]) * dev[0] + ny[k] * dev[1]) - nz[k] * dev[2];
        const float s2 = ora_dot3(res, nrm) < 0.0f ? -1.0f : 1.0f;
        const float se = s2 * eps;
        float* r = aoRays + 8 * (pix * R + z);
        r[0] = pos[0] + se * nrm[0];
        r[1] = pos[1] + se * nrm[1];
        r[2] = pos[2] + se * nrm[2];
        r[3] = 0.0f;
        r[4] = res[0]; r[5] = res[1]; r[6] = res[2];
        r[7] = aoMaxRadius;
      }
    }
}

/* kernel_TraceAORay (closest-hit variant, attenuation 0) summed over the
 * samples and kernel_AO2Color (examples/02_rtao/rtao.cpp:62-73,167-185):
 * visibility = number of unoccluded samples, colour = grey of
 * powf(visibility / R, power) quantised to 8 bits; 0 for pixels without a hit.
 * aoHit: one flag per (pixel, sample). */
void ora_rtao_colors(const float* positions, const uint8_t* aoHit, uint64_t nPix, uint32_t R, float power,
                     float* visibility, uint32_t* colors)
{
  for (uint64_t p = 0; p < nPix; p++)
  {
    const int hit = positions[4 * p + 1] < 10000000.0f;
    float vis = 0.0f;
    if (hit)
      for (uint32_t z = 0; z < R; z++) vis = vis + (aoHit[p * R + z] ? 0.0f : 1.0f);
    visibility[p] = vis;
    if (!hit)
    {
      colors[p] = 0u;
      continue;
    }
    const float normCoeff = 1.0f / (float)(1u * R);
    const float a = vis * normCoeff;
    const float res = powf(a, power);
    const float c = fmin_lm(fmax_lm(res, 0.0f), 1.0f) * 255.0f;
    const float c1 = fmin_lm(fmax_lm(1.0f, 0.0f), 1.0f) * 255.0f;
    const int g = ora_f2i(c), w = ora_f2i(c1);
    colors[p] = (uint32_t)(g + (g << 8) + (g << 16) + (int)((uint32_t)w << 24));
  }
}
