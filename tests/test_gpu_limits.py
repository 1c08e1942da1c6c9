"""The largest geometry the formats hold: 2^24 - 1 triangles, the top of the
24-bit leaf-start field (core/raytrace_common.h:38-51).  Built in the binary
layout, every stage checked and hits bit-exact against the oracle, hits
reaching the top of the sorted order; the benchmark's 4-wide tree (cubic
grid, largest-first collapse, FP16 nodes) held to the stated tolerance; one
triangle more is refused with HRT_ERR_CAPACITY before anything is built."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF
N_MAX = (1 << 24) - 1


def test_largest_geometry(native):
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    v, idx = wl.soup(97, N_MAX, off=0.0005)
    # rays aimed at the centroids of random triangles (each ~0.001 across),
    # and rays through the soup from a sphere around it
    rays = np.concatenate([wl.rays_at_triangles(98, v, idx, 200000), wl.sphere_rays(99, 50000)])
    o = orc.OracleBVH(v, idx)
    assert o.status == 0 and o.n_tris == N_MAX
    want = o.trace(rays)
    want_any = o.trace(rays, any_hit=True)
    hit = want["geomId"] != MISS
    assert hit.mean() > 0.2
    assert int(want["primId"][hit].max()) >= N_MAX - 200000  # leaf starts near the top of the field

    s = SceneRT()
    gid = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
    s.AddInstance(gid)
    s.CommitScene()
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_MORTON_SORTED).reshape(-1, 2), o.morton_sorted())
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_RUN_STARTS), o.run_starts())
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_LR_COUNTS), o.lr_counts())
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_PRIM_INDICES), o.prim_indices())
    np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32).reshape(-1, 8),
                                  np.ascontiguousarray(want).view(np.uint32).reshape(-1, 8))
    np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), want_any)
    s.close()

    t = SceneRT(layout="bvh4_f16")
    t.set_bvh4_merge(1)
    t.set_morton_frame(E.MORTON_CUBIC)
    t.set_bvh4_collapse(E.BVH4_COLLAPSE_LARGEST_FIRST)
    gid = t.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
    t.AddInstance(gid)
    t.CommitScene()
    g = t.RayQuery_NearestHit(rays).view(np.uint32).reshape(-1, 8).copy()
    w = np.ascontiguousarray(want).view(np.uint32).reshape(-1, 8).copy()
    hg, hw = g[:, 3] != MISS, w[:, 3] != MISS
    np.testing.assert_array_equal(hg, hw)
    g[hg, 1] = t.export(gid, E.EXPORT_PRIM_INDICES)[g[hg, 1]]
    w[hw, 1] = o.prim_indices()[w[hw, 1]]
    same = g[:, 1] == w[:, 1]
    np.testing.assert_array_equal(g[same], w[same])
    tg = g[~same, 0].view(np.float32).astype(np.float64)
    tw = w[~same, 0].view(np.float32).astype(np.float64)
    assert np.all(np.abs(tg - tw) <= 1e-5 * np.abs(tw))
    assert np.count_nonzero(~same) <= max(2, g.shape[0] // 100000)
    np.testing.assert_array_equal(t.RayQuery_AnyHit(rays), want_any)
    t.close()
    o.close()

    # one triangle more than the leaf-start field can address
    big = np.concatenate([idx, idx[:3]])
    u = SceneRT()
    with pytest.raises(E.HrtError) as ei:
        u.AddGeom_Triangles3f(v, v.shape[0], big, big.size, vByteStride=16)
    assert ei.value.status == E.HRT_ERR_CAPACITY
    u.close()
