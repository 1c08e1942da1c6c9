"""Generate the golden vectors in tests/golden/ from HeavyRT's own CPU code.

Runs the reference checker (oracle/_ref/ref_harness, compiled from the
reference sources by oracle/Makefile.ref) on small seeded scenes and stores
inputs and outputs in golden_*.npz.  The reference ships no golden vectors of
its own for this path, so these fixtures are the pinned record of what its
LBVH builder and BVH2CommonRT traversal produce.

    python tests/golden/make_golden.py      (needs the reference sources)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from heavyrt_gb300 import native_build, workload as wl  # noqa: E402
from oracle import oracle as orc  # noqa: E402

OUT = Path(__file__).resolve().parent


def cases():
    # triangle soups across the size thresholds of the reference builder:
    # centroid vs box-centre Morton input below/above 256 triangles
    # (core/builders/lbvh.cpp:279) and the 256/2048-node perfect top tree
    # switch at 8192 triangles (core/builders/lbvh.cpp:90)
    for n in (1, 3, 200, 300, 8193):
        v, idx = wl.soup(1000 + n, n)
        rays = wl.camera_rays((0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0, 48, 48)
        rays = np.concatenate([rays, wl.sphere_rays(77 + n, 256, 3.0),
                               wl.rays_at_triangles(78 + n, v, idx, 512, jitter=0.01)])
        yield f"soup{n}", v, idx, rays
    # heightfield: equal Morton codes -> multi-triangle leaves
    v, idx, _ = wl.heightfield(5, 24, 24)
    rays = wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 64, 36)
    yield "heightfield24", v, idx, rays
    # duplicated triangles: long runs of one code, ties in t between leaf members
    base_v, base_i = wl.soup(4242, 40, off=0.3)
    v = np.concatenate([base_v] * 5)
    idx = np.concatenate([base_i + k * base_v.shape[0] for k in range(5)]).astype(np.uint32)
    rays = wl.rays_at_triangles(91, v, idx, 1024, jitter=0.05)
    yield "duplicates40x5", v, idx, rays
    # indexed mesh with shared vertices and stride-free float4 input
    v, idx, _ = wl.heightfield(6, 8, 5)
    rays = wl.rays_at_triangles(92, v, idx, 256)
    rays[:, 3] = 0.5  # tNear > 0
    yield "heightfield8x5_tnear", v, idx, rays


def perspective(fov_deg, aspect, near, far):
    t = 1.0 / np.tan(np.radians(fov_deg) / 2.0)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = t / aspect, t
    m[2, 2], m[2, 3], m[3, 2] = (far + near) / (near - far), 2.0 * far * near / (near - far), -1.0
    return m


def look_at(eye, target, up):
    eye, target, up = (np.asarray(x, np.float64) for x in (eye, target, up))
    f = (target - eye) / np.linalg.norm(target - eye)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m


def eye_ray_cases():
    """Inverse projection / world-view matrices for the renderers' eye-ray set-up:
    the heightfield camera, and two perturbed (non-affine) matrix pairs."""
    p = np.linalg.inv(perspective(60.0, 16.0 / 9.0, 0.01, 100.0)).astype(np.float32)
    v = np.linalg.inv(look_at((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1))).astype(np.float32)
    yield p, v, 160, 90, 0.0, 3.4028234663852886e38
    rng = np.random.default_rng(1)
    for w, h in ((33, 17), (64, 64)):
        yield ((p + rng.normal(0, 0.05, (4, 4))).astype(np.float32), (v + rng.normal(0, 0.05, (4, 4))).astype(np.float32),
               w, h, 0.5, 7.0)


def make_eye_rays():
    """raygen_eye.npz: the reference's own eye-ray set-up (oracle/_ref/raygen_harness)."""
    out = {}
    for k, (p, v, w, h, tn, tf) in enumerate(eye_ray_cases()):
        rays = orc.reference_eye_rays(p, v, w, h, tn, tf)
        out.update({f"proj_inv{k}": p, f"world_view_inv{k}": v, f"size{k}": np.array([w, h]),
                    f"range{k}": np.array([tn, tf], np.float32), f"rays{k}": rays})
        print("eye rays", k, w, h)
    np.savez_compressed(OUT / "raygen_eye.npz", **out)


def main():
    native_build.build_all()
    if orc.reference_harness() is None:
        raise SystemExit("reference sources not available: cannot regenerate golden vectors")
    make_eye_rays()
    for name, v, idx, rays in cases():
        ref = orc.run_reference(v, idx, rays)
        np.savez_compressed(
            OUT / f"golden_{name}.npz",
            verts=v, idx=idx, rays=rays,
            scene_box=ref["scene_box"],
            morton_unsorted=ref["morton_unsorted"], morton_sorted=ref["morton_sorted"],
            compressed=ref["compressed"], run_starts=ref["run_starts"],
            lr_nodes=ref["lr_nodes"].view(np.uint32), lr_counts=ref["lr_counts"],
            peach_nodes=ref["peach_nodes"].view(np.uint32), prim_indices=ref["prim_indices"],
            sorted_indices=ref["sorted_indices"],
            hits=ref["hits"].view(np.uint32), any=ref["any"],
            ref_counters=np.array([ref["trace_info"]["avgNC"], ref["trace_info"]["avgTC"], ref["trace_info"]["avgBLB"]]),
        )
        print(name, v.shape[0], idx.size // 3, rays.shape[0], int((ref["hits"]["geomId"] != 0xFFFFFFFF).sum()))


if __name__ == "__main__":
    main()
