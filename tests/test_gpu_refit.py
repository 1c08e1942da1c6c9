"""UpdateGeom_Triangles3f: a refit (BUILD_REFIT) keeps the tree's topology
and sorted order and gives, for every ray, the hit a fresh build of the moved
vertices gives (same triangle, t, u, v); a rebuild replaces the geometry."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF


def _scene(v, idx, layout=0, merge=None, tlas_instances=None):
    from heavyrt_gb300 import SceneRT

    s = SceneRT(layout=layout)
    if merge is not None:
        s.set_bvh4_merge(merge)
    g = s.AddGeom_Triangles3f(v, len(v), idx, idx.size, vByteStride=16)
    for m in (tlas_instances or [np.eye(4, dtype=np.float32)]):
        s.AddInstance(g, m)
    s.CommitScene()
    return s, g


def _by_original(s, g, hits):
    """Hits with primId mapped to the original triangle index."""
    from heavyrt_gb300 import engine as E

    h = hits.view(np.uint32).reshape(-1, 8).copy()
    prim = s.export(g, E.EXPORT_PRIM_INDICES)
    m = h[:, 1] != MISS
    h[m, 1] = prim[h[m, 1]]
    return h


def _moved(seed):
    """A heightfield and its animated version (same triangles, new heights),
    and a soup whose triangles each move by a small random offset."""
    from heavyrt_gb300 import workload as wl

    v0, idx, _ = wl.heightfield(seed, 90, 80)
    v1 = v0.copy()
    v1[:, 2] += 0.05 * np.sin(7.0 * v0[:, 0]) * np.cos(5.0 * v0[:, 1])
    s0, si = wl.soup(seed + 1, 20000, off=0.02)
    s1 = s0.copy()
    rng = np.random.default_rng(seed)
    s1[:, :3] += np.repeat(rng.uniform(-0.05, 0.05, (20000, 3)), 3, axis=0).astype(np.float32)
    return [(v0, v1, idx), (s0, s1, si)]


def _rays(v, idx, seed):
    from heavyrt_gb300 import workload as wl

    r = np.concatenate([wl.rays_at_triangles(seed, v, idx, 6000, jitter=0.02), wl.sphere_rays(seed, 2000)])
    r[::5, 3] = 0.3
    return r


@pytest.mark.parametrize("layout,merge", [(0, None), (2, 1), (1, 0), (3, 4)])
def test_refit_equals_fresh_build(native, layout, merge):
    from heavyrt_gb300 import BUILD_REFIT
    from heavyrt_gb300 import engine as E

    for v0, v1, idx in _moved(3):
        s, g = _scene(v0, idx, layout, merge)
        prim_before = s.export(g, E.EXPORT_PRIM_INDICES)
        s.UpdateGeom_Triangles3f(g, v1, len(v1), idx, idx.size, BUILD_REFIT, 16)
        with pytest.raises(E.HrtError):
            s.RayQuery_NearestHit(_rays(v1, idx, 1)[:10])  # not committed yet
        s.CommitScene()
        np.testing.assert_array_equal(s.export(g, E.EXPORT_PRIM_INDICES), prim_before)  # order kept
        fresh, fg = _scene(v1, idx, layout, merge)
        rays = _rays(v1, idx, 2)
        got = _by_original(s, g, s.RayQuery_NearestHit(rays))
        want = _by_original(fresh, fg, fresh.RayQuery_NearestHit(rays))
        diff = np.any(got != want, axis=1)
        assert np.array_equal(got[diff, 0], want[diff, 0]) and diff.sum() <= 2  # only exact ties may differ
        assert (got[:, 1] != MISS).sum() > 3000
        np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), fresh.RayQuery_AnyHit(rays))
        box = s.GetGeomBoxes()[0]
        np.testing.assert_array_equal(box[:3], v1[:, :3].min(axis=0))
        np.testing.assert_array_equal(box[4:7], v1[:, :3].max(axis=0))


def test_refit_boxes_contain_children_and_triangles(native):
    from heavyrt_gb300 import BUILD_REFIT
    from heavyrt_gb300 import engine as E

    v0, v1, idx = _moved(5)[1]
    s, g = _scene(v0, idx)
    s.UpdateGeom_Triangles3f(g, v1, len(v1), idx, idx.size, BUILD_REFIT, 16)
    lr = s.export(g, E.EXPORT_LR_NODES)
    L = (len(lr) + 1) // 2
    lo, hi = lr["boxMin"], lr["boxMax"]
    for i in range(L - 1):
        for c in (lr["leftOffset"][i], lr["escapeIndex"][i]):
            assert np.all(lo[i] <= lo[c]) and np.all(hi[i] >= hi[c])
    si = s.export(g, E.EXPORT_SORTED_INDICES).reshape(-1, 3)
    runs = s.export(g, E.EXPORT_RUN_STARTS)
    ends = np.r_[runs[1:], len(si)]
    p = v1[:, :3]
    for k in range(L):
        tri = p[si[runs[k]:ends[k]].reshape(-1)]
        np.testing.assert_array_equal(lo[L - 1 + k], tri.min(axis=0))
        np.testing.assert_array_equal(hi[L - 1 + k], tri.max(axis=0))


def test_refit_batch_geometry_and_instances(native):
    from heavyrt_gb300 import BUILD_REFIT, SceneRT

    geoms = _moved(7)
    s = SceneRT()
    ids = s.add_geoms_batched([g[0] for g in geoms], [g[2] for g in geoms])
    mats = []
    for k in range(6):
        m = np.eye(4, dtype=np.float32)
        m[:3, 3] = [3.0 * k, 0.0, 0.0]
        mats.append(m)
    for k, m in enumerate(mats):
        s.AddInstance(ids[k % 2], m)
    s.CommitScene()
    for (v0, v1, idx), g in zip(geoms, ids):
        s.UpdateGeom_Triangles3f(g, v1, len(v1), idx, idx.size, BUILD_REFIT, 16)
    s.CommitScene()
    fresh = SceneRT()
    fids = [fresh.AddGeom_Triangles3f(v1, len(v1), idx, idx.size, vByteStride=16) for _, v1, idx in geoms]
    for k, m in enumerate(mats):
        fresh.AddInstance(fids[k % 2], m)
    fresh.CommitScene()
    from heavyrt_gb300 import workload as wl

    rays = wl.sphere_rays(3, 20000, 12.0)
    a, b = s.RayQuery_NearestHit(rays), fresh.RayQuery_NearestHit(rays)
    np.testing.assert_array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))
    np.testing.assert_array_equal(a["instId"], b["instId"])
    np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), fresh.RayQuery_AnyHit(rays))


def test_rebuild_replaces_geometry(native):
    from heavyrt_gb300 import BUILD_HIGH
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    v0, i0 = wl.soup(1, 3000)
    v1, i1 = wl.soup(2, 7000)  # another size
    s, g = _scene(v0, i0)
    s.UpdateGeom_Triangles3f(g, v1, len(v1), i1, i1.size, BUILD_HIGH, 16)
    s.CommitScene()
    rays = _rays(v1, i1, 4)
    np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32),
                                  orc.OracleBVH(v1, i1).trace(rays).view(np.uint32))
    with pytest.raises(E.HrtError) as ei:  # a refit must keep the counts
        s.UpdateGeom_Triangles3f(g, v0, len(v0), i0, i0.size, 3, 16)
    assert ei.value.status == E.HRT_ERR_INVALID_ARGUMENT
    with pytest.raises(E.HrtError):
        s.UpdateGeom_Triangles3f(99, v0, len(v0), i0, i0.size, BUILD_HIGH, 16)
