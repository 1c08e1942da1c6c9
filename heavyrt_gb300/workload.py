"""Seeded synthetic scenes and rays (heavyrt_gb300/csrc/workload.c) and the
benchmark configurations built from them.

Configurations (HeavyRT publishes no scenes for this path; these stand in for
its eye-ray and RTAO renderers' inputs):
  config0: 65,536-triangle soup (centres U[-1,1]^3, vertex offsets U[-0.02,0.02]^3),
           pinhole at (0,0,3) looking down -z, +y up, 60 deg vertical FOV,
           512 x 512 eye rays, tmin 0, tmax 1e9.
  config1: 1024 x 1024-quad heightfield (2,097,152 triangles) over [-1,1]^2,
           eye rays 1920 x 1080 from (0,-2.5,1.5) at the origin (60 deg, +z up),
           16 cosine-weighted AO rays per primary hit, length 0.1 x scene
           diagonal, origin offset 1e-4 along the normal, any-hit.
  config2: two scenes traced separately, each with 2M eye rays that all hit
           and 16 AO rays per hit (33,177,600): the config1 heightfield seen
           from (0,0,2) straight down (30 deg), and an 8,388,608-triangle soup
           (vertex offsets U[-0.005,0.005]^3) seen from (0,0,3) (30 deg).
  config3: 256 soups of log-uniform size, see config3().
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_BUILD = Path(__file__).resolve().parent / "_build"
_lib = None

SEED_SOUP = 0x5EED0001
SEED_HEIGHTFIELD = 0x5EED0002
SEED_AO = 0x5EED0003
SEED_BATCH = 0x5EED0004


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        p = _BUILD / "libhrt_workload.so"
        if not p.exists():
            raise RuntimeError(f"workload generator not built ({p} missing): run __graft_entry__.build()")
        L = C.CDLL(str(p))
        vp, u32, u64, f32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float
        L.hrt_wl_pcg32.argtypes = [u64, u64, u32, vp]
        L.hrt_wl_soup.argtypes = [u64, u32, f32, f32, f32, vp, vp]
        L.hrt_wl_heightfield.argtypes = [u64, u32, u32, vp, vp, vp]
        L.hrt_wl_camera_rays.argtypes = [vp, vp, vp, f32, u32, u32, f32, f32, vp]
        L.hrt_wl_sphere_rays.argtypes = [u64, u32, f32, vp]
        L.hrt_wl_ao_rays.argtypes = [u64, u64, vp, vp, vp, vp, u32, f32, f32, vp, vp]
        L.hrt_wl_ao_rays.restype = u64
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def pcg32(seed: int, stream: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint32)
    lib().hrt_wl_pcg32(seed, stream, n, _p(out))
    return out


def soup(seed: int, n_tris: int, lo: float = -1.0, hi: float = 1.0, off: float = 0.02):
    v = np.empty((3 * n_tris, 4), dtype=np.float32)
    idx = np.empty(3 * n_tris, dtype=np.uint32)
    lib().hrt_wl_soup(seed, n_tris, lo, hi, off, _p(v), _p(idx))
    return v, idx


def heightfield(seed: int, nx: int, ny: int):
    v = np.empty(((nx + 1) * (ny + 1), 4), dtype=np.float32)
    idx = np.empty(6 * nx * ny, dtype=np.uint32)
    params = np.empty(24, dtype=np.float64)
    lib().hrt_wl_heightfield(seed, nx, ny, _p(v), _p(idx), _p(params))
    return v, idx, params


def camera_rays(eye, target, up, fov_deg: float, width: int, height: int, tmin: float = 0.0, tmax: float = 1e9):
    e = np.asarray(eye, dtype=np.float32)
    t = np.asarray(target, dtype=np.float32)
    u = np.asarray(up, dtype=np.float32)
    rays = np.empty((width * height, 8), dtype=np.float32)
    lib().hrt_wl_camera_rays(_p(e), _p(t), _p(u), fov_deg, width, height, tmin, tmax, _p(rays))
    return rays


def perspective(fov_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """OpenGL-style projection matrix (row-major 4x4, float64)."""
    t = 1.0 / np.tan(np.radians(fov_deg) / 2.0)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = t / aspect, t
    m[2, 2], m[2, 3], m[3, 2] = (far + near) / (near - far), 2.0 * far * near / (near - far), -1.0
    return m


def look_at(eye, target, up) -> np.ndarray:
    """World-to-view matrix of a camera at eye looking at target (row-major 4x4, float64)."""
    eye, target, up = (np.asarray(x, np.float64) for x in (eye, target, up))
    f = (target - eye) / np.linalg.norm(target - eye)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m


def camera_inverses(eye, target, up, fov_deg: float, width: int, height: int):
    """(projInv, worldViewInv) as float32 row-major 4x4, the renderers' camera inputs."""
    p = np.linalg.inv(perspective(fov_deg, width / height, 0.01, 100.0)).astype(np.float32)
    v = np.linalg.inv(look_at(eye, target, up)).astype(np.float32)
    return p, v


def vertex_normals(verts: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """Area-weighted vertex normals (float4, w = 0) of an indexed mesh."""
    p = np.asarray(verts, np.float64).reshape(-1, 4)[:, :3]
    t = np.asarray(idx, np.int64).reshape(-1, 3)
    fn = np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]])
    n = np.zeros_like(p)
    for k in range(3):
        np.add.at(n, t[:, k], fn)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    return np.concatenate([n, np.zeros((n.shape[0], 1))], axis=1).astype(np.float32)


def sphere_rays(seed: int, n: int, radius: float = 3.0):
    rays = np.empty((n, 8), dtype=np.float32)
    lib().hrt_wl_sphere_rays(seed, n, radius, _p(rays))
    return rays


def rays_at_triangles(seed: int, verts: np.ndarray, idx: np.ndarray, n: int, radius: float = 3.0,
                      jitter: float = 0.0) -> np.ndarray:
    """Rays from random points on a sphere toward the centroids of random
    triangles (optionally jittered), so that most of them hit something."""
    rng = np.random.default_rng(seed)
    v = np.asarray(verts, dtype=np.float64).reshape(-1, 4)[:, :3]
    tri = np.asarray(idx, dtype=np.int64).reshape(-1, 3)
    pick = rng.integers(0, tri.shape[0], size=n)
    c = v[tri[pick]].mean(axis=1) + rng.uniform(-jitter, jitter, size=(n, 3))
    z = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    s = np.sqrt(1 - z * z)
    o = radius * np.stack([s * np.cos(ph), s * np.sin(ph), z], axis=1)
    d = c - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), dtype=np.float32)
    rays[:, 0:3] = o
    rays[:, 4:7] = d
    rays[:, 7] = 1e9
    return rays


def ao_rays(seed: int, eye_rays: np.ndarray, hits: np.ndarray, verts: np.ndarray, sorted_idx: np.ndarray,
            per_hit: int, length: float, offset: float = 1e-4):
    """AO rays from primary hits (CRT_Hit records, sorted-order primIds)."""
    eye_rays = np.ascontiguousarray(eye_rays, dtype=np.float32)
    hits_u = np.ascontiguousarray(hits).view(np.uint32).reshape(-1, 8)
    n_hit = int(np.count_nonzero(hits_u[:, 3] != 0xFFFFFFFF))
    out = np.empty((n_hit * per_hit, 8), dtype=np.float32)
    owner = np.empty(n_hit * per_hit, dtype=np.uint32)
    v = np.ascontiguousarray(verts, dtype=np.float32)
    si = np.ascontiguousarray(sorted_idx, dtype=np.uint32)
    w = lib().hrt_wl_ao_rays(seed, eye_rays.shape[0], _p(eye_rays), _p(hits_u), _p(v), _p(si), per_hit, length, offset,
                             _p(out), _p(owner))
    assert w == out.shape[0]
    return out, owner


@dataclass
class Workload:
    name: str
    verts: np.ndarray
    idx: np.ndarray
    eye_rays: np.ndarray
    params: dict = field(default_factory=dict)


def config0() -> Workload:
    v, idx = soup(SEED_SOUP, 65536, -1.0, 1.0, 0.02)
    rays = camera_rays((0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0, 512, 512, 0.0, 1e9)
    return Workload("soup65536_eye512", v, idx, rays, {"tris": 65536, "width": 512, "height": 512, "seed": SEED_SOUP})


def config1(nx: int = 1024, width: int = 1920, height: int = 1080) -> Workload:
    v, idx, hp = heightfield(SEED_HEIGHTFIELD, nx, nx)
    rays = camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, width, height, 0.0, 1e9)
    lo = v[:, :3].min(axis=0)
    hi = v[:, :3].max(axis=0)
    diag = float(np.linalg.norm(hi.astype(np.float64) - lo.astype(np.float64)))
    return Workload(f"heightfield{nx}x{nx}_eye{width}x{height}_ao16", v, idx, rays,
                    {"tris": 2 * nx * nx, "width": width, "height": height, "seed": SEED_HEIGHTFIELD,
                     "ao_per_hit": 16, "ao_length": 0.1 * diag, "ao_offset": 1e-4, "ao_seed": SEED_AO,
                     "heightfield_params": hp.tolist()})


SEED_SOUP_8M = 0x5EED0006


def config2(scene: str, width: int = 1920, height: int = 1080, soup_tris: int = 8388608) -> Workload:
    """One scene of the quantised-node precision configuration: "heightfield"
    (config1's mesh) or "soup" (soup_tris triangles, offsets +-0.005).  The
    30-degree cameras keep every eye ray on the mesh, so 16 AO rays per hit
    make 16 x width x height AO rays."""
    if scene == "heightfield":
        v, idx, _ = heightfield(SEED_HEIGHTFIELD, 1024, 1024)
        eye, name = (0.0, 0.0, 2.0), "heightfield1024x1024"
    elif scene == "soup":
        v, idx = soup(SEED_SOUP_8M, soup_tris, -1.0, 1.0, 0.005)
        eye, name = (0.0, 0.0, 3.0), f"soup{soup_tris}"
    else:
        raise ValueError(scene)
    rays = camera_rays(eye, (0, 0, 0), (0, 1, 0), 30.0, width, height, 0.0, 1e9)
    lo = v[:, :3].min(axis=0)
    hi = v[:, :3].max(axis=0)
    diag = float(np.linalg.norm(hi.astype(np.float64) - lo.astype(np.float64)))
    return Workload(f"{name}_eye{width}x{height}_ao16", v, idx, rays,
                    {"tris": int(idx.size // 3), "width": width, "height": height, "eye": list(eye), "fov": 30.0,
                     "ao_per_hit": 16, "ao_length": 0.1 * diag, "ao_offset": 1e-4, "ao_seed": SEED_AO})


def frame_ao_rays(w: Workload, hits: np.ndarray, sorted_idx: np.ndarray):
    """The AO rays of a workload's frame from its eye hits (CRT_Hit records of
    a one-instance scene, sorted-order primIds) and the geometry's sorted index
    buffer."""
    p = w.params
    ao, _ = ao_rays(p["ao_seed"], w.eye_rays, hits, w.verts, sorted_idx, p["ao_per_hit"], p["ao_length"],
                    p["ao_offset"])
    return ao


def log_uniform_counts(seed: int, stream: int, n: int, lo: int, hi: int) -> np.ndarray:
    """n integers log-uniform in [lo, hi]: floor(lo * (hi/lo)^u), u = (pcg32 >> 8) * 2^-24."""
    u = (pcg32(seed, stream, n) >> 8).astype(np.float64) * 2.0 ** -24
    c = np.floor(lo * np.exp(u * np.log(hi / lo))).astype(np.int64)
    return np.clip(c, lo, hi)


@dataclass
class BatchWorkload:
    name: str
    verts: list              # per scene: float32 [3N, 4]
    idx: list                # per scene: uint32 [3N]
    rays: np.ndarray         # all scenes' rays, scene after scene: float32 [R, 8]
    ray_offsets: np.ndarray  # uint32 [S+1]: scene s owns rays ray_offsets[s] .. ray_offsets[s+1]-1
    params: dict = field(default_factory=dict)


def config3(n_scenes: int = 256, tri_lo: int = 1024, tri_hi: int = 262144, ray_lo: int = 4096, ray_hi: int = 65536,
            seed: int = SEED_BATCH) -> BatchWorkload:
    """Many independent soups (generator of config0) with log-uniform triangle
    and ray counts; each scene's rays start uniformly on the sphere of radius 3
    and aim at uniform points of [-1,1]^3."""
    tris = log_uniform_counts(seed, 1, n_scenes, tri_lo, tri_hi)
    nrays = log_uniform_counts(seed, 2, n_scenes, ray_lo, ray_hi)
    verts, idx, rays = [], [], []
    for i in range(n_scenes):
        v, ix = soup(seed + 16 + i, int(tris[i]), -1.0, 1.0, 0.02)
        verts.append(v)
        idx.append(ix)
        rays.append(sphere_rays(seed + 65536 + i, int(nrays[i]), 3.0))
    offs = np.zeros(n_scenes + 1, dtype=np.uint32)
    offs[1:] = np.cumsum(nrays)
    return BatchWorkload(f"soups{n_scenes}_tris{tri_lo}-{tri_hi}_rays{ray_lo}-{ray_hi}", verts, idx,
                         np.ascontiguousarray(np.concatenate(rays)), offs,
                         {"scenes": n_scenes, "tris": int(tris.sum()), "rays": int(nrays.sum()), "seed": seed,
                          "tri_counts": tris.tolist(), "ray_counts": nrays.tolist()})


def scene_file(path, verts: np.ndarray, idx: np.ndarray):
    """Write the HRTSCN01 container read by the reference checker harness."""
    v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 4)
    i = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1)
    with open(path, "wb") as f:
        f.write(b"HRTSCN01")
        f.write(np.array([v.shape[0], i.size], dtype=np.uint64).tobytes())
        f.write(v.tobytes())
        f.write(i.tobytes())


def ray_file(path, rays: np.ndarray):
    r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    with open(path, "wb") as f:
        f.write(b"HRTRAY01")
        f.write(np.array([r.shape[0]], dtype=np.uint64).tobytes())
        f.write(r.tobytes())
