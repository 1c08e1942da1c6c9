"""The oracle (C restatement of HeavyRT's LBVH build + BVH2CommonRT traversal)
against the golden vectors produced by HeavyRT's own code, and against that
code live where its sources are present.  CPU only."""
import numpy as np
import pytest

from conftest import GOLDEN, golden_cases


def _load(case):
    return dict(np.load(GOLDEN / f"golden_{case}.npz"))


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_build_matches_golden(host_libs, case):
    from oracle import oracle as orc

    g = _load(case)
    o = orc.OracleBVH(g["verts"], g["idx"])
    assert o.status == 0
    np.testing.assert_array_equal(o.scene_box().view(np.uint32), g["scene_box"].view(np.uint32))
    np.testing.assert_array_equal(o.morton_unsorted(), g["morton_unsorted"])
    np.testing.assert_array_equal(o.morton_sorted(), g["morton_sorted"])
    np.testing.assert_array_equal(o.compressed(), g["compressed"])
    np.testing.assert_array_equal(o.run_starts(), g["run_starts"])
    np.testing.assert_array_equal(o.lr_nodes().view(np.uint32), g["lr_nodes"])
    np.testing.assert_array_equal(o.lr_counts(), g["lr_counts"])
    np.testing.assert_array_equal(o.peach_nodes().view(np.uint32), g["peach_nodes"])
    np.testing.assert_array_equal(o.prim_indices(), g["prim_indices"])
    np.testing.assert_array_equal(o.sorted_indices(), g["sorted_indices"])


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_trace_matches_golden(host_libs, case):
    from oracle import oracle as orc

    g = _load(case)
    o = orc.OracleBVH(g["verts"], g["idx"])
    hits, (pairs, tris), _ = o.trace(g["rays"], counters=True, threads=1)
    np.testing.assert_array_equal(hits.view(np.uint32).reshape(-1, 8), g["hits"].reshape(-1, 8))
    anyh = o.trace(g["rays"], any_hit=True)
    np.testing.assert_array_equal(anyh, g["any"])
    # HeavyRT's own counters (core/BVH2CommonRT.cpp:68-69,125): 2 nodes per pair, BLB = 64 B/pair + 60 B/triangle
    n = g["rays"].shape[0]
    avg_nc, avg_tc, avg_blb = g["ref_counters"]
    assert abs(2.0 * pairs / n - avg_nc) < 1e-3
    assert abs(tris / n - avg_tc) < 1e-3
    assert abs((64.0 * pairs + 60.0 * tris) / n - avg_blb) < 1e-2


def test_anyhit_is_nearest_found(host_libs):
    """Any-hit semantics (HeavyRT siblings, core/BVH2CommonRTStacklessLBVH.cpp:161-165):
    true exactly when the nearest-hit traversal accepts some triangle."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    v, idx, _ = wl.heightfield(11, 48, 48)
    rays = np.concatenate([wl.rays_at_triangles(5, v, idx, 4000, jitter=0.05), wl.sphere_rays(6, 4000)])
    rays[::3, 7] = 0.05  # short rays: some hits fall beyond tFar
    o = orc.OracleBVH(v, idx)
    hits = o.trace(rays)
    anyh = o.trace(rays, any_hit=True)
    np.testing.assert_array_equal(anyh, hits["geomId"] != 0xFFFFFFFF)


def test_oracle_flags_leaf_overflow(host_libs):
    """More than 127 triangles with one Morton code overflow the reference's
    7-bit leaf count (core/raytrace_common.h:40,48-51); the oracle flags it."""
    from oracle import oracle as orc

    tri = np.array([[0, 0, 0, 1], [1, 0, 0, 1], [0, 1, 0, 1]], dtype=np.float32)
    v = np.concatenate([tri] * 200 + [tri + np.array([5, 5, 5, 0], np.float32)])
    idx = np.arange(v.shape[0], dtype=np.uint32)
    o = orc.OracleBVH(v, idx)
    assert o.status == 1


REF_CASES = [("soup", 2), ("soup", 17), ("soup", 4096), ("soup", 9000), ("soup", 30000), ("hf", 32), ("hf", 128)]


@pytest.mark.parametrize("kind,n", REF_CASES)
def test_oracle_matches_reference_live(host_libs, kind, n):
    """Bit-exact against the reference's own builder and traversal, compiled
    from its sources (skipped where they are absent)."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    if orc.reference_harness() is None:
        pytest.skip("reference sources not present on this machine")
    if kind == "soup":
        v, idx = wl.soup(300 + n, n)
    else:
        v, idx, _ = wl.heightfield(300 + n, n, n)
    rays = np.concatenate([wl.rays_at_triangles(n, v, idx, 2000, jitter=0.02), wl.sphere_rays(n, 500)])
    ref = orc.run_reference(v, idx, rays)
    o = orc.OracleBVH(v, idx)
    np.testing.assert_array_equal(o.morton_unsorted(), ref["morton_unsorted"])
    np.testing.assert_array_equal(o.morton_sorted(), ref["morton_sorted"])
    np.testing.assert_array_equal(o.lr_nodes().view(np.uint32), ref["lr_nodes"].view(np.uint32))
    np.testing.assert_array_equal(o.lr_counts(), ref["lr_counts"])
    np.testing.assert_array_equal(o.peach_nodes().view(np.uint32), ref["peach_nodes"].view(np.uint32))
    np.testing.assert_array_equal(o.prim_indices(), ref["prim_indices"])
    np.testing.assert_array_equal(o.trace(rays).view(np.uint32), ref["hits"].view(np.uint32))
    np.testing.assert_array_equal(o.trace(rays, any_hit=True), ref["any"])


def _eye_cases():
    z = np.load(GOLDEN / "raygen_eye.npz")
    k = 0
    while f"rays{k}" in z:
        yield (z[f"proj_inv{k}"], z[f"world_view_inv{k}"], *[int(x) for x in z[f"size{k}"]],
               *[float(x) for x in z[f"range{k}"]], z[f"rays{k}"])
        k += 1


def test_eye_rays_restatement_matches_reference_fixture(host_libs):
    """The renderers' eye-ray set-up restated in C equals the reference's own
    helpers (examples/render_common.h, compiled against the LiteMath stand-in)."""
    from oracle import oracle as orc

    for p, v, w, h, tn, tf, want in _eye_cases():
        got = orc.eye_rays(p, v, w, h, tn, tf)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
        live = orc.reference_eye_rays(p, v, w, h, tn, tf)
        if live is not None:
            np.testing.assert_array_equal(live.view(np.uint32), want.view(np.uint32))
