"""Generate the golden vectors in tests/golden/ from HeavyRT's own CPU code.

Runs the reference checkers (oracle/_ref/ref_harness, raygen_harness and
render_harness, compiled from the reference sources by oracle/Makefile.ref) on
small seeded scenes and stores inputs and outputs in golden_*.npz,
raygen_eye.npz and render_frames.npz.  The reference ships no golden vectors of
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


perspective, look_at = wl.perspective, wl.look_at


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


vertex_normals = wl.vertex_normals


def render_cases():
    """Frames of the two example renderers over a 48x48 heightfield: a packed-order
    image (sides multiples of 8) and a row-order one with a z range and a
    non-identity normal matrix."""
    v, idx, _ = wl.heightfield(7, 48, 48)
    nrm = vertex_normals(v, idx)
    wv = np.linalg.inv(look_at((0.3, -1.7, 1.0), (0, 0, -0.1), (0, 0, 1))).astype(np.float32)
    yield dict(name="a", verts=v, idx=idx, normals=nrm, width=64, height=48, z_near=0.0, z_far=3.4028234663852886e38,
               rays_per_pixel=4, radius=0.3, power=1.0, norm_matrix=np.eye(4, dtype=np.float32),
               proj_inv=np.linalg.inv(perspective(60.0, 64 / 48, 0.01, 100.0)).astype(np.float32), world_view_inv=wv)
    yield dict(name="b", verts=v, idx=idx, normals=nrm, width=37, height=21, z_near=0.5, z_far=3.0,
               rays_per_pixel=16, radius=0.1, power=1.0, norm_matrix=np.diag([1.0, 2.0, 0.5, 1.0]).astype(np.float32),
               proj_inv=np.linalg.inv(perspective(50.0, 37 / 21, 0.01, 100.0)).astype(np.float32), world_view_inv=wv)


def make_render():
    """render_frames.npz: the example renderers' own frame kernels (oracle/_ref/render_harness)."""
    import hashlib
    out = {}
    q = orc.reference_render("qmc", None, None, None, None, 0, 0, rays_per_pixel=4)
    out["qmc_table"] = q["qmc"]
    for r in (1, 3, 4, 16):
        t = orc.reference_render("qmc", None, None, None, None, 0, 0, rays_per_pixel=r)["tile"]
        out[f"tile_sha256_r{r}"] = np.frombuffer(hashlib.sha256(t.tobytes()).digest(), np.uint8)
    for c in render_cases():
        k = c["name"]
        common = dict(verts=c["verts"], idx=c["idx"], proj_inv=c["proj_inv"], world_view_inv=c["world_view_inv"],
                      width=c["width"], height=c["height"])
        ref = orc.reference_render("rtao", normals=c["normals"], z_near=c["z_near"], z_far=c["z_far"],
                                   rays_per_pixel=c["rays_per_pixel"], radius=c["radius"], power=c["power"],
                                   norm_matrix=c["norm_matrix"], **common)
        hit = ref["positions"][:, 1] < orc.AO_HIT_BACK
        sel = np.repeat(hit, c["rays_per_pixel"])
        for name in ("verts", "idx", "normals"):  # one scene for both frames
            out[name] = c[name]
        for name in ("proj_inv", "world_view_inv", "norm_matrix"):
            out[f"{k}_{name}"] = c[name]
        out[f"{k}_params"] = np.array([c["width"], c["height"], c["rays_per_pixel"]], np.uint32)
        out[f"{k}_fparams"] = np.array([c["z_near"], c["z_far"], c["radius"], c["power"]], np.float32)
        out[f"{k}_positions"] = ref["positions"]
        out[f"{k}_ao_rays"] = ref["ao_rays"][sel]
        out[f"{k}_ao_hit"] = ref["ao_hit"][sel]
        out[f"{k}_visibility"] = np.where(hit, ref["visibility"], 0.0).astype(np.float32)
        out[f"{k}_colors"] = ref["colors"]
        if c["width"] % 8 == 0 and c["height"] % 8 == 0:  # the eye renderer's packing needs it
            e = orc.reference_render("eye", **common)
            out[f"{k}_eye_packed"] = e["packed"]
            out[f"{k}_eye_colors"] = e["colors"]
        print("render", k, c["width"], c["height"], int(hit.sum()), int(ref["ao_hit"][sel].sum()))
    np.savez_compressed(OUT / "render_frames.npz", **out)


def main():
    native_build.build_all()
    if orc.reference_harness() is None:
        raise SystemExit("reference sources not available: cannot regenerate golden vectors")
    make_eye_rays()
    make_render()
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
