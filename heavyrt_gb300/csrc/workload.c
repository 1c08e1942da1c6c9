/*
 * Seeded synthetic scenes and rays with the shapes of HeavyRT's benchmark
 * cases: random triangle soups, a sum-of-sines heightfield, pinhole eye rays
 * and cosine-weighted ambient-occlusion rays.  HeavyRT's own scenes (Hydra XML
 * / VSGF meshes) are not used; these generators stand in for them.
 *
 * Random numbers: PCG32 (O'Neill, "PCG: A Family of Simple Fast Space-Efficient
 * Statistically Good Algorithms for Random Number Generation", 2014), the
 * XSH-RR output function with the 64-bit LCG multiplier 6364136223846793005.
 * A uniform float in [0,1) is (next() >> 8) * 2^-24.
 *
 * Geometry is computed in double and rounded once to float, so the output does
 * not depend on the host's float libm.  Vertices are float4 with w = 1, rays
 * are interleaved {posAndNear, dirAndFar} float4 pairs as HeavyRT's
 * RayQuery_* take them (core/CrossRT.h:143,151).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct
{
  uint64_t state, inc;
} wl_pcg;

static uint32_t wl_next(wl_pcg* r)
{
  const uint64_t old = r->state;
  r->state = old * 6364136223846793005ULL + r->inc;
  const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  const uint32_t rot = (uint32_t)(old >> 59u);
  return (xs >> rot) | (xs << ((-rot) & 31u));
}

static void wl_seed(wl_pcg* r, uint64_t seed, uint64_t stream)
{
  r->state = 0u;
  r->inc = (stream << 1u) | 1u;
  wl_next(r);
  r->state += seed;
  wl_next(r);
}

static double wl_uniform(wl_pcg* r) { return (double)(wl_next(r) >> 8) * (1.0 / 16777216.0); }
static double wl_range(wl_pcg* r, double lo, double hi) { return lo + (hi - lo) * wl_uniform(r); }

/* Raw PCG32 output, exposed so the tests can check the generator against the
 * published reference sequence. */
void hrt_wl_pcg32(uint64_t seed, uint64_t stream, uint32_t n, uint32_t* out)
{
  wl_pcg r;
  wl_seed(&r, seed, stream);
  for (uint32_t i = 0; i < n; i++) out[i] = wl_next(&r);
}

/* Non-indexed triangle soup: centre ~ U[lo,hi]^3, each vertex = centre +
 * U[-off,off]^3.  verts: 3*nTris float4, idx: 3*nTris (0..3n-1). */
void hrt_wl_soup(uint64_t seed, uint32_t nTris, float lo, float hi, float off, float* verts, uint32_t* idx)
{
  wl_pcg r;
  wl_seed(&r, seed, 1);
  for (uint32_t t = 0; t < nTris; t++)
  {
    const double c[3] = {wl_range(&r, lo, hi), wl_range(&r, lo, hi), wl_range(&r, lo, hi)};
    for (int v = 0; v < 3; v++)
    {
      float* p = verts + 4 * (3 * (size_t)t + v);
      for (int k = 0; k < 3; k++) p[k] = (float)(c[k] + wl_range(&r, -off, off));
      p[3] = 1.0f;
      idx[3 * (size_t)t + v] = 3 * t + v;
    }
  }
}

/* Heightfield of nx*ny quads over [-1,1]^2:
 *   z(x,y) = sum_{k<8} (0.1 / 2^k) * sin(a_k x + b_k y + phi_k)
 * with |(a_k,b_k)| = pi * 2^k * U[1,2], direction U[0,2pi), phi_k U[0,2pi).
 * verts: (nx+1)(ny+1) float4; idx: 6*nx*ny, quad (i,j) -> (v00,v10,v11),(v00,v11,v01).
 * params (optional, 24 doubles): a_k, b_k, phi_k as drawn. */
void hrt_wl_heightfield(uint64_t seed, uint32_t nx, uint32_t ny, float* verts, uint32_t* idx, double* params)
{
  wl_pcg r;
  wl_seed(&r, seed, 2);
  double a[8], b[8], ph[8];
  for (int k = 0; k < 8; k++)
  {
    const double mag = 3.14159265358979323846 * (double)(1u << k) * wl_range(&r, 1.0, 2.0);
    const double ang = wl_range(&r, 0.0, 2.0 * 3.14159265358979323846);
    a[k] = mag * cos(ang);
    b[k] = mag * sin(ang);
    ph[k] = wl_range(&r, 0.0, 2.0 * 3.14159265358979323846);
    if (params) { params[3 * k + 0] = a[k]; params[3 * k + 1] = b[k]; params[3 * k + 2] = ph[k]; }
  }
  for (uint32_t j = 0; j <= ny; j++)
    for (uint32_t i = 0; i <= nx; i++)
    {
      const double x = -1.0 + 2.0 * (double)i / (double)nx;
      const double y = -1.0 + 2.0 * (double)j / (double)ny;
      double z = 0.0;
      for (int k = 0; k < 8; k++) z += (0.1 / (double)(1u << k)) * sin(a[k] * x + b[k] * y + ph[k]);
      float* p = verts + 4 * ((size_t)j * (nx + 1) + i);
      p[0] = (float)x;
      p[1] = (float)y;
      p[2] = (float)z;
      p[3] = 1.0f;
    }
  size_t w = 0;
  for (uint32_t j = 0; j < ny; j++)
    for (uint32_t i = 0; i < nx; i++)
    {
      const uint32_t v00 = j * (nx + 1) + i, v10 = v00 + 1, v01 = v00 + (nx + 1), v11 = v01 + 1;
      idx[w++] = v00; idx[w++] = v10; idx[w++] = v11;
      idx[w++] = v00; idx[w++] = v11; idx[w++] = v01;
    }
}

static void wl_norm(double v[3])
{
  const double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= l; v[1] /= l; v[2] /= l;
}

/* Normalised in float: each component divided by the length. */
static void wl_normf(float v[3])
{
  const float l = sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
  v[0] = v[0] / l;
  v[1] = v[1] / l;
  v[2] = v[2] / l;
}

static float wl_uniformf(wl_pcg* r) { return (float)(wl_next(r) >> 8) * (1.0f / 16777216.0f); }

static void wl_cross(const double a[3], const double b[3], double o[3])
{
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

/* Pinhole camera at eye looking at target, `up` hint, vertical field of view
 * fovDeg; one normalised ray per pixel centre, row 0 at the top.  The frame
 * (forward, right, up, tan of the half angle, aspect) is set up in double and
 * rounded once to float; each pixel's direction then takes only correctly
 * rounded float operations in a fixed order, so the device generator
 * (hrt_gen_pinhole_rays) makes the same rays bit for bit. */
void hrt_wl_camera_rays(const float eye[3], const float target[3], const float up[3], float fovDeg, uint32_t width,
                        uint32_t height, float tmin, float tmax, float* rays)
{
  double f[3] = {target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]};
  wl_norm(f);
  const double u0[3] = {up[0], up[1], up[2]};
  double rgt[3], u[3];
  wl_cross(f, u0, rgt);
  wl_norm(rgt);
  wl_cross(rgt, f, u);
  const float ff[3] = {(float)f[0], (float)f[1], (float)f[2]};
  const float fr[3] = {(float)rgt[0], (float)rgt[1], (float)rgt[2]};
  const float fu[3] = {(float)u[0], (float)u[1], (float)u[2]};
  const float th = (float)tan(0.5 * (double)fovDeg * 3.14159265358979323846 / 180.0);
  const float aspect = (float)((double)width / (double)height);
  for (uint32_t y = 0; y < height; y++)
    for (uint32_t x = 0; x < width; x++)
    {
      const float sx = ((2.0f * ((float)x + 0.5f)) / (float)width - 1.0f) * th * aspect;
      const float sy = (1.0f - (2.0f * ((float)y + 0.5f)) / (float)height) * th;
      float d[3];
      for (int k = 0; k < 3; k++) d[k] = (ff[k] + sx * fr[k]) + sy * fu[k];
      wl_normf(d);
      float* r = rays + 8 * ((size_t)y * width + x);
      r[0] = eye[0]; r[1] = eye[1]; r[2] = eye[2]; r[3] = tmin;
      r[4] = d[0]; r[5] = d[1]; r[6] = d[2]; r[7] = tmax;
    }
}

/* Random rays for a scene: origin uniform on the sphere of radius `radius`
 * about the origin, direction toward a uniform point of [-1,1]^3.
 * rays: n*8 floats, tmin = 0, tmax = 1e9. */
void hrt_wl_sphere_rays(uint64_t seed, uint32_t n, float radius, float* rays)
{
  wl_pcg r;
  wl_seed(&r, seed, 3);
  for (uint32_t i = 0; i < n; i++)
  {
    const double z = wl_range(&r, -1.0, 1.0);
    const double phi = wl_range(&r, 0.0, 2.0 * 3.14159265358979323846);
    const double s = sqrt(1.0 - z * z);
    const double o[3] = {radius * s * cos(phi), radius * s * sin(phi), radius * z};
    const double t[3] = {wl_range(&r, -1.0, 1.0), wl_range(&r, -1.0, 1.0), wl_range(&r, -1.0, 1.0)};
    double d[3] = {t[0] - o[0], t[1] - o[1], t[2] - o[2]};
    wl_norm(d);
    float* ry = rays + 8 * (size_t)i;
    ry[0] = (float)o[0]; ry[1] = (float)o[1]; ry[2] = (float)o[2]; ry[3] = 0.0f;
    ry[4] = (float)d[0]; ry[5] = (float)d[1]; ry[6] = (float)d[2]; ry[7] = 1e9f;
  }
}

/* Ambient-occlusion rays from primary hits.  hits: CRT_Hit records (32 bytes:
 * t, primId, instId, geomId, coords[4]) for the eye rays; the hit triangle's
 * vertex ids are sortedIdx[3*primId .. 3*primId+2] (the index buffer in the
 * BVH's sorted order, as HeavyRT returns sorted primIds).  For every hit,
 * `perHit` cosine-weighted directions about the geometric normal turned toward
 * the eye (Malley's method: a uniform point of the unit disk, by rejection
 * from the square, lifted to the hemisphere; basis of Duff et al., "Building
 * an Orthonormal Basis, Revisited", 2017); origin = hit point + offset *
 * normal; tmin = 0, tmax = length.  Float arithmetic with correctly rounded
 * operations only, in a fixed order, so the device generator
 * (hrt_gen_ao_rays) makes the same rays bit for bit.  Each hit draws from its
 * own PCG stream (seed, eye-ray index + 16), so the output does not depend on
 * how the loop is split.  Returns the number of rays written; aoRays needs
 * room for perHit * (number of hits) rays; owner (optional) receives the
 * eye-ray index of each AO ray. */
uint64_t hrt_wl_ao_rays(uint64_t seed, uint64_t nEye, const float* eyeRays, const uint32_t* hits, const float* verts,
                        const uint32_t* sortedIdx, uint32_t perHit, float length, float offset, float* aoRays,
                        uint32_t* owner)
{
  uint64_t w = 0;
  for (uint64_t i = 0; i < nEye; i++)
  {
    const uint32_t* h = hits + 8 * i;
    if (h[3] == 0xFFFFFFFFu) continue; /* geomId == -1: miss */
    float t;
    memcpy(&t, &h[0], 4);
    const float* er = eyeRays + 8 * i;
    const float p[3] = {er[0] + t * er[4], er[1] + t * er[5], er[2] + t * er[6]};
    const uint32_t prim = h[1];
    const float* A = verts + 4 * (size_t)sortedIdx[3 * (size_t)prim + 0];
    const float* B = verts + 4 * (size_t)sortedIdx[3 * (size_t)prim + 1];
    const float* C = verts + 4 * (size_t)sortedIdx[3 * (size_t)prim + 2];
    const float e1[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
    const float e2[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
    float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    wl_normf(n);
    if ((n[0] * er[4] + n[1] * er[5]) + n[2] * er[6] > 0.0f) { n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2]; }
    const float sgn = n[2] >= 0.0f ? 1.0f : -1.0f;
    const float aa = -1.0f / (sgn + n[2]);
    const float bb = (n[0] * n[1]) * aa;
    const float tx[3] = {1.0f + ((sgn * n[0]) * n[0]) * aa, sgn * bb, -(sgn * n[0])};
    const float ty[3] = {bb, sgn + (n[1] * n[1]) * aa, -n[1]};
    const float o[3] = {p[0] + offset * n[0], p[1] + offset * n[1], p[2] + offset * n[2]};
    wl_pcg r;
    wl_seed(&r, seed, i + 16);
    for (uint32_t s = 0; s < perHit; s++)
    {
      float x = 0.0f, y = 0.0f, rr = 0.0f;
      for (int tries = 0; tries < 64; tries++)
      {
        x = 2.0f * wl_uniformf(&r) - 1.0f;
        y = 2.0f * wl_uniformf(&r) - 1.0f;
        rr = x * x + y * y;
        if (rr <= 1.0f) break;
      }
      if (rr > 1.0f) { x = 0.0f; y = 0.0f; rr = 0.0f; } /* probability (1 - pi/4)^64 */
      const float z = sqrtf(1.0f - rr);
      float d[3];
      for (int k = 0; k < 3; k++) d[k] = (x * tx[k] + y * ty[k]) + z * n[k];
      wl_normf(d);
      float* ry = aoRays + 8 * w;
      ry[0] = o[0]; ry[1] = o[1]; ry[2] = o[2]; ry[3] = 0.0f;
      ry[4] = d[0]; ry[5] = d[1]; ry[6] = d[2]; ry[7] = length;
      if (owner) owner[w] = (uint32_t)i;
      w++;
    }
  }
  return w;
}
