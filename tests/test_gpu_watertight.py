"""The watertight triangle test (HRT_OPTION_TRIANGLE_TEST = HRT_TRI_WATERTIGHT)
against the oracle's restatement of it (oracle/hrt_oracle.c leaf_test_wt:
Woop, Benthin & Wald 2013 with exact FP32 edge-function signs).  The binary
layout makes the reference's traversal decisions, so with the same triangle
test its results equal the oracle's bit for bit; the 4-wide layouts differ
only at ties within 1e-5 relative t.  Also: no ray aimed at a shared edge or
vertex of a closed surface passes through it, and the scene's other paths
(instances, batches, refit, blobs, launch shapes, short stacks) keep the test."""
import numpy as np
import pytest

from conftest import GOLDEN, golden_cases

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF
LAYOUTS = [("bvh2", None), ("bvh4", 1), ("bvh4_f16", 1), ("bvh4_q8", 1), ("bvh4", 0)]


def _scene(v, idx, layout="bvh2", merge=None, instances=None):
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E

    s = SceneRT(layout=layout, triangle_test=E.TRI_WATERTIGHT)
    if merge is not None:
        s.set_bvh4_merge(merge)
    gid = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
    for m in instances if instances is not None else [None]:
        s.AddInstance(gid, m)
    s.CommitScene()
    return s, gid


def _u32(h):
    return np.ascontiguousarray(h).view(np.uint32).reshape(-1, 8)


def _compare(got, want, layout, tie_limit=True):
    g, w = _u32(got), _u32(want)
    if layout == "bvh2":
        np.testing.assert_array_equal(g, w)
        return
    np.testing.assert_array_equal(g[:, 3] != MISS, w[:, 3] != MISS)
    same = g[:, 1] == w[:, 1]
    np.testing.assert_array_equal(g[same], w[same])
    tg = g[~same, 0].view(np.float32).astype(np.float64)
    tw = w[~same, 0].view(np.float32).astype(np.float64)
    assert np.all(np.abs(tg - tw) <= 1e-5 * np.abs(tw))
    if tie_limit:
        assert np.count_nonzero(~same) <= max(2, g.shape[0] // 100000)


def _heightfield_edge_rays(v, nx):
    """Vertical rays from above, aimed exactly at every grid vertex and at the
    midpoint of every grid edge of an nx x nx heightfield (the points where
    two or more triangles meet)."""
    xy = v[:, :2].reshape(nx + 1, nx + 1, 2).astype(np.float32)
    pts = [xy.reshape(-1, 2),
           (0.5 * (xy[:, 1:] + xy[:, :-1])).reshape(-1, 2),
           (0.5 * (xy[1:, :] + xy[:-1, :])).reshape(-1, 2),
           (0.5 * (xy[1:, 1:] + xy[:-1, :-1])).reshape(-1, 2)]
    p = np.concatenate(pts).astype(np.float32)
    rays = np.zeros((p.shape[0], 8), np.float32)
    rays[:, 0:2] = p
    rays[:, 2] = 3.0
    rays[:, 6] = -1.0
    rays[:, 7] = 1e9
    # interior points only (the outer border has one triangle side)
    lo, hi = float(v[:, 0].min()), float(v[:, 0].max())
    inside = (p[:, 0] > lo) & (p[:, 0] < hi) & (p[:, 1] > lo) & (p[:, 1] < hi)
    return rays[inside]


@pytest.mark.parametrize("case", golden_cases())
def test_watertight_golden_scenes_vs_oracle(native, case):
    from oracle import oracle as orc

    g = dict(np.load(GOLDEN / f"golden_{case}.npz"))
    o = orc.OracleBVH(g["verts"], g["idx"])
    want = o.trace(g["rays"], watertight=True)
    want_any = o.trace(g["rays"], any_hit=True, watertight=True)
    for layout, merge in LAYOUTS:
        s, _ = _scene(g["verts"], g["idx"], layout, merge)
        _compare(s.RayQuery_NearestHit(g["rays"]), want, layout)
        np.testing.assert_array_equal(s.RayQuery_AnyHit(g["rays"]), want_any, err_msg=f"{case} {layout}")
        s.close()


def test_watertight_config0_vs_oracle_every_layout_and_shape(native):
    """C0 (65,536-triangle soup, 512 x 512 eye rays) plus rays at random
    triangles, every layout, persistent pool and one thread per ray, short
    stacks of 4..64 shared entries."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    w = wl.config0()
    rays = np.concatenate([w.eye_rays, wl.rays_at_triangles(5, w.verts, w.idx, 20000, jitter=0.01)])
    o = orc.OracleBVH(w.verts, w.idx)
    want = o.trace(rays, watertight=True)
    want_any = o.trace(rays, any_hit=True, watertight=True)
    assert (want["geomId"] != MISS).mean() > 0.3
    for layout, merge in LAYOUTS:
        s, _ = _scene(w.verts, w.idx, layout, merge)
        for persistent, stack in ((1, 0), (0, 0), (1, 4), (0, 16), (1, 64)):
            for kind in (0, 1):
                s.set_trace_config(kind, 128, persistent, 16, 24, stack)
            _compare(s.RayQuery_NearestHit(rays), want, layout)
            np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), want_any, err_msg=layout)
        s.close()


def test_watertight_heightfield_edges_never_leak(native):
    """A closed heightfield: every vertical ray aimed exactly at a shared
    vertex or edge hits it under the watertight test, on the GPU and in the
    oracle, with equal results."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    nx = 128
    v, idx, _ = wl.heightfield(77, nx, nx)
    rays = _heightfield_edge_rays(v, nx)
    assert rays.shape[0] > 60000
    o = orc.OracleBVH(v, idx)
    want = o.trace(rays, watertight=True)
    assert np.all(want["geomId"] != MISS)
    for layout, merge in LAYOUTS[:3]:
        s, _ = _scene(v, idx, layout, merge)
        got = s.RayQuery_NearestHit(rays)
        assert np.all(got["geomId"] != MISS), layout
        # rays aimed at shared edges and vertices tie between the triangles
        # that meet there; the 4-wide order may pick another of them
        _compare(got, want, layout, tie_limit=False)
        assert s.RayQuery_AnyHit(rays).all()
        s.close()


def test_watertight_instances_two_level_equals_instance_loop(native):
    """Transformed instances under the watertight test: the instance-tree
    kernel gives the hits of the instance-by-instance traversal."""
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(31, 3000, off=0.05)
    rng = np.random.default_rng(4)
    mats = []
    for k in range(5):
        m = np.eye(4, dtype=np.float32)
        a = rng.uniform(0, 2 * np.pi)
        m[:2, :2] = [[np.cos(a), -np.sin(a)], [np.sin(a), np.cos(a)]]
        m[:3, 3] = rng.uniform(-1.5, 1.5, 3)
        mats.append(m)
    rays = wl.sphere_rays(8, 20000, 4.0)
    res = {}
    for tlas in (1, 0):
        s = SceneRT(triangle_test=E.TRI_WATERTIGHT, layout="bvh4_f16")
        s.set_tlas(bool(tlas))
        gid = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
        for m in mats:
            s.AddInstance(gid, m)
        s.CommitScene()
        res[tlas] = (_u32(s.RayQuery_NearestHit(rays)), s.RayQuery_AnyHit(rays))
        s.close()
    (a, aa), (b, bb) = res[1], res[0]
    np.testing.assert_array_equal(aa, bb)
    assert (a[:, 3] != MISS).sum() > 1000
    diff = np.any(a != b, axis=1)
    np.testing.assert_array_equal(a[diff, 0], b[diff, 0])  # only exact ties between instances may differ
    assert diff.sum() <= 2


def test_watertight_batch_refit_and_blob(native, tmp_path):
    """Segmented batch build and query, refit after moved vertices, and a blob
    round trip keep the watertight records; a blob of the other test is
    refused."""
    import torch

    from heavyrt_gb300 import HrtError, SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    scenes = [wl.soup(600 + k, n, off=0.03) for k, n in enumerate((700, 5000, 1))]
    rays = [wl.rays_at_triangles(k, v, i, 3000, jitter=0.02) for k, (v, i) in enumerate(scenes)]
    s = SceneRT(triangle_test=E.TRI_WATERTIGHT)
    ids = s.add_geoms_batched([v for v, _ in scenes], [i for _, i in scenes])
    for g in ids:
        s.AddInstance(g)
    s.CommitScene()
    allr = np.concatenate(rays)
    offs = np.zeros(len(rays) + 1, np.uint32)
    offs[1:] = np.cumsum([len(r) for r in rays])
    dr, do = torch.from_numpy(allr).cuda(), torch.from_numpy(offs.view(np.int32)).cuda()
    ds = torch.from_numpy(np.arange(len(ids), dtype=np.int32)).cuda()
    out = torch.zeros((len(allr), 8), dtype=torch.int32, device="cuda")
    s.query_multi(E.query_desc(0, dr.data_ptr(), len(allr), out.data_ptr(), do.data_ptr(), ds.data_ptr(), len(ids)))
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    for k, (v, i) in enumerate(scenes):
        want = _u32(orc.OracleBVH(v, i).trace(rays[k], watertight=True)).copy()
        hit = want[:, 1] != MISS
        want[hit, 2] = k
        want[hit, 3] = ids[k]
        np.testing.assert_array_equal(got[offs[k]:offs[k + 1]], want)
    s.close()

    # refit: moved vertices, same triangles -> the hits of a fresh build
    v, i = scenes[1]
    moved = v.copy()
    moved[:, :3] += np.random.default_rng(2).uniform(-0.01, 0.01, (v.shape[0], 3)).astype(np.float32)
    s, gid = _scene(v, i, "bvh4_f16", 1)
    s.UpdateGeom_Triangles3f(gid, moved, moved.shape[0], i, i.size, E.BUILD_REFIT, 16)
    s.CommitScene()
    fresh, _ = _scene(moved, i, "bvh4_f16", 1)
    a, b = _u32(s.RayQuery_NearestHit(rays[1])), _u32(fresh.RayQuery_NearestHit(rays[1]))
    np.testing.assert_array_equal(a[:, 0], b[:, 0])
    np.testing.assert_array_equal(s.RayQuery_AnyHit(rays[1]), fresh.RayQuery_AnyHit(rays[1]))
    fresh.close()

    # blob round trip, and refusal by a scene of the other triangle test
    path = tmp_path / "wt.blob"
    s.save_geom(gid, path)
    want = _u32(s.RayQuery_NearestHit(rays[1]))
    s.close()
    r, _ = _scene(v[:3], i[:3], "bvh4_f16", 1)
    gid2 = r.load_geom(path)
    r.ClearScene()
    r.AddInstance(gid2)
    r.CommitScene()
    want[want[:, 3] != MISS, 3] = gid2  # the restored geometry's id in this scene
    np.testing.assert_array_equal(_u32(r.RayQuery_NearestHit(rays[1])), want)
    r.close()
    mt = SceneRT(layout="bvh4_f16")
    with pytest.raises(HrtError, match="triangle test"):
        mt.load_geom(path)
    # the option is refused once a geometry exists
    mt.AddGeom_Triangles3f(v, v.shape[0], i, i.size, vByteStride=16)
    with pytest.raises(HrtError):
        mt.set_triangle_test(E.TRI_WATERTIGHT)
    mt.close()
