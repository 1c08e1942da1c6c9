"""Batched scenes: the segmented build gives every geometry exactly the arrays
of its own single build, segmented queries give every ray exactly the hit of a
per-scene query, captured graphs replay the same launches, and the autotuner
changes no result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF
EXPORTS = range(0, 9)  # scene box .. unsorted codes (every LBVH stage)


def _geoms():
    """Geometries of the edge sizes: empty, 1-3 triangles, both sides of the
    256-triangle centroid rule, a tile boundary, runs of equal codes."""
    from heavyrt_gb300 import workload as wl

    out = []
    for i, n in enumerate([1, 0, 2, 3, 255, 256, 257, 4096, 4097, 9000]):
        v, idx = wl.soup(500 + i, n, off=0.05) if n else (np.zeros((0, 4), np.float32), np.zeros(0, np.uint32))
        out.append((v, idx))
    v, idx, _ = wl.heightfield(33, 60, 45)  # many multi-triangle leaves
    out.append((v, idx))
    # 40 copies of 5 triangles: long runs of equal codes
    v5, i5 = wl.soup(7, 5, off=0.05)
    out.append((np.concatenate([v5] * 40), np.concatenate([i5 + 15 * k for k in range(40)]).astype(np.uint32)))
    # shared vertices with unreferenced extra vertices widening the box
    v, idx, _ = wl.heightfield(34, 20, 20)
    extra = np.array([[5.0, -3.0, 2.0, 1.0], [-4.0, 6.0, -1.0, 1.0]], np.float32)
    out.append((np.concatenate([v, extra]), idx))
    return out


def _single(v, idx, layout=0, merge=None):
    from heavyrt_gb300 import SceneRT

    s = SceneRT(layout=layout)
    if merge is not None:
        s.set_bvh4_merge(merge)
    gid = s.AddGeom_Triangles3f(np.ascontiguousarray(v, np.float32), len(v), idx, idx.size, vByteStride=16)
    s.AddInstance(gid)
    s.CommitScene()
    return s, gid


def _batched(geoms, layout=0, merge=None, prefix=None):
    from heavyrt_gb300 import SceneRT

    s = SceneRT(layout=layout)
    if merge is not None:
        s.set_bvh4_merge(merge)
    if prefix is not None:  # a geometry added one at a time before the batch
        s.AddGeom_Triangles3f(prefix[0], len(prefix[0]), prefix[1], prefix[1].size, vByteStride=16)
    ids = s.add_geoms_batched([g[0] for g in geoms], [g[1] for g in geoms])
    for gid in ids:
        s.AddInstance(gid)
    s.CommitScene()
    return s, ids


def _same_exports(a, ga, b, gb, whats):
    for what in whats:
        x, y = a.export(ga, what), b.export(gb, what)
        assert x.dtype == y.dtype and x.shape == y.shape, what
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8), err_msg=f"export {what}")


def test_batch_build_equals_single_builds(native):
    from heavyrt_gb300 import workload as wl

    geoms = _geoms()
    pv, pi = wl.soup(99, 300, off=0.05)
    s, ids = _batched(geoms, prefix=(pv, pi))
    assert ids == list(range(1, len(geoms) + 1)) and s.GetGeomNum() == len(geoms) + 1
    for (v, idx), gid in zip(geoms, ids):
        info = s.geom_info(gid)
        assert info["tris"] == idx.size // 3
        if idx.size == 0:
            assert info["leaves"] == 0
            continue
        ref, rg = _single(v, idx)
        assert info["leaves"] == ref.geom_info(rg)["leaves"] and info["pairs"] == ref.geom_info(rg)["pairs"]
        _same_exports(s, gid, ref, rg, [w for w in EXPORTS if w != 0])
        np.testing.assert_array_equal(s.export(gid, 0).view(np.uint32), ref.export(rg, 0).view(np.uint32))
    boxes = s.GetGeomBoxes()
    assert boxes.shape == (len(geoms) + 1, 8)
    s.ClearGeom()
    assert s.GetGeomNum() == 0


def test_batch_build_matches_oracle(native):
    """The oracle directly (not only through the single build) on two geometries."""
    from heavyrt_gb300 import engine as E
    from oracle import oracle as orc

    geoms = _geoms()
    s, ids = _batched(geoms)
    for k in (4, 10):
        v, idx = geoms[k]
        o = orc.OracleBVH(v, idx)
        gid = ids[k]
        np.testing.assert_array_equal(s.export(gid, E.EXPORT_MORTON_SORTED).reshape(-1, 2), o.morton_sorted())
        np.testing.assert_array_equal(s.export(gid, E.EXPORT_RUN_STARTS), o.run_starts())
        np.testing.assert_array_equal(s.export(gid, E.EXPORT_LR_NODES).view(np.uint32).reshape(-1),
                                      np.asarray(o.lr_nodes()).view(np.uint32).reshape(-1))
        np.testing.assert_array_equal(s.export(gid, E.EXPORT_PRIM_INDICES), o.prim_indices())


def _segment_rays(geoms, order, per=600):
    """Rays for segments tracing instances `order` (ids; may repeat, may be out
    of range); an empty segment sits in the middle."""
    from heavyrt_gb300 import workload as wl

    rays, offs = [], [0]
    for j, inst in enumerate(order):
        if j == len(order) // 2:
            offs.append(offs[-1])  # empty segment
        if inst < len(geoms) and geoms[inst][1].size:
            v, idx = geoms[inst]
            r = np.concatenate([wl.rays_at_triangles(j, v, idx, per, jitter=0.03), wl.sphere_rays(j, per // 3)])
        else:
            r = wl.sphere_rays(j, per // 2)
        r[::5, 3] = 0.5  # some rays with tNear > 0
        rays.append(r)
        offs.append(offs[-1] + len(r))
    seg_inst = list(order)
    seg_inst.insert(len(order) // 2, 0)
    return np.ascontiguousarray(np.concatenate(rays)), np.array(offs, np.uint32), np.array(seg_inst, np.uint32)


def _run_multi(s, rays, offs, seg_inst, kind):
    import torch

    from heavyrt_gb300 import engine as E

    dr = torch.from_numpy(rays).cuda()
    do = torch.from_numpy(offs.view(np.int32)).cuda()
    ds = torch.from_numpy(seg_inst.view(np.int32)).cuda()
    out = torch.zeros((len(rays), 8) if kind == 0 else (len(rays),), dtype=torch.int32 if kind == 0 else torch.uint8,
                      device="cuda")
    d = E.query_desc(kind, dr.data_ptr(), len(rays), out.data_ptr(), do.data_ptr(), ds.data_ptr(), len(seg_inst))
    s.query_multi(d, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    res = out.cpu().numpy()
    return res.view(np.uint32) if kind == 0 else res.astype(bool)


def _expected(geoms, singles, rays, offs, seg_inst, geom_ids):
    """Per-segment hits from single-scene queries (singles: geometry index ->
    scene), instId rewritten to the segment's instance (instance i holds
    geometry i) and geomId to the batch's geometry id."""
    want = np.zeros((len(rays), 8), np.uint32)
    want_any = np.zeros(len(rays), bool)
    for k in range(len(seg_inst)):
        a, b = offs[k], offs[k + 1]
        if a == b:
            continue
        r = rays[a:b]
        inst = int(seg_inst[k])
        if inst not in singles:  # out of range or empty geometry: misses
            want[a:b, 0] = r[:, 7].view(np.uint32)
            want[a:b, 1:4] = MISS
            continue
        h = singles[inst].RayQuery_NearestHit(r).view(np.uint32).reshape(-1, 8).copy()
        hit = h[:, 1] != MISS
        h[hit, 2] = inst
        h[hit, 3] = geom_ids[inst]
        want[a:b] = h
        want_any[a:b] = singles[inst].RayQuery_AnyHit(r)
    return want, want_any


@pytest.mark.parametrize("layout,merge", [(0, None), (2, 1), (1, 0), (3, 8)])
def test_segmented_query_equals_per_scene_queries(native, layout, merge):
    geoms = _geoms()
    s, ids = _batched(geoms, layout=layout, merge=merge)
    singles = {}
    for gi, (v, idx) in enumerate(geoms):
        if idx.size:
            singles[gi] = _single(v, idx, layout, merge)[0]
    if layout != 0:  # the batch's 4-wide nodes are the single builds' nodes
        from heavyrt_gb300 import engine as E

        for gi in singles:
            _same_exports(s, ids[gi], singles[gi], 0, [E.EXPORT_NODES4])
    order = [3, 0, 9, 1, 12, 4, len(geoms) + 5, 10, 3, 11, 7, 2, 6, 8, 5]
    rays, offs, seg_inst = _segment_rays(geoms, order)
    got = _run_multi(s, rays, offs, seg_inst, 0)
    got_any = _run_multi(s, rays, offs, seg_inst, 1)
    want, want_any = _expected(geoms, singles, rays, offs, seg_inst, ids)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(got_any, want_any)
    assert got[:, 1].tolist().count(MISS) < len(rays)  # the rays do hit


def test_segmented_query_vs_oracle(native):
    """Rays of each segment against the oracle of that segment's geometry."""
    from oracle import oracle as orc

    geoms = _geoms()
    s, ids = _batched(geoms)
    order = [10, 4, 8]
    rays, offs, seg_inst = _segment_rays(geoms, order, per=900)
    got = _run_multi(s, rays, offs, seg_inst, 0)
    got_any = _run_multi(s, rays, offs, seg_inst, 1)
    for k in range(len(seg_inst)):
        a, b = offs[k], offs[k + 1]
        if a == b:
            continue
        inst = int(seg_inst[k])
        o = orc.OracleBVH(*geoms[inst])
        w = o.trace(rays[a:b]).view(np.uint32).reshape(-1, 8).copy()
        hit = w[:, 1] != MISS
        w[hit, 2] = inst
        w[hit, 3] = ids[inst]
        np.testing.assert_array_equal(got[a:b], w)
        np.testing.assert_array_equal(got_any[a:b], o.trace(rays[a:b], any_hit=True))


def test_graph_replays_queries(native):
    import torch

    from heavyrt_gb300 import engine as E

    geoms = _geoms()
    s, ids = _batched(geoms)
    rays, offs, seg_inst = _segment_rays(geoms, [4, 9, 10, 2])
    dr = torch.from_numpy(rays).cuda()
    do = torch.from_numpy(offs.view(np.int32)).cuda()
    ds = torch.from_numpy(seg_inst.view(np.int32)).cuda()
    hits = torch.zeros((len(rays), 8), dtype=torch.int32, device="cuda")
    anyo = torch.zeros(len(rays), dtype=torch.uint8, device="cuda")
    d0 = E.query_desc(0, dr.data_ptr(), len(rays), hits.data_ptr(), do.data_ptr(), ds.data_ptr(), len(seg_inst))
    d1 = E.query_desc(1, dr.data_ptr(), len(rays), anyo.data_ptr(), do.data_ptr(), ds.data_ptr(), len(seg_inst))
    plain = torch.zeros((len(rays), 8), dtype=torch.int32, device="cuda")
    d2 = E.query_desc(0, dr.data_ptr(), len(rays), plain.data_ptr())  # unsegmented: all instances
    g = s.capture([d0, d1, d2])
    stream = torch.cuda.current_stream().cuda_stream
    want = _run_multi(s, rays, offs, seg_inst, 0)
    want_any = _run_multi(s, rays, offs, seg_inst, 1)
    for _ in range(3):
        hits.zero_()
        anyo.zero_()
        g.launch(stream)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(hits.cpu().numpy().view(np.uint32), want)
        np.testing.assert_array_equal(anyo.cpu().numpy().astype(bool), want_any)
    np.testing.assert_array_equal(plain.cpu().numpy().view(np.uint32), s.RayQuery_NearestHit(rays).view(np.uint32).reshape(-1, 8))
    # new ray contents in the same buffers: the replay traces them
    rays2 = rays.copy()
    rays2[:, 7] = 0.25  # short rays
    dr.copy_(torch.from_numpy(rays2))
    g.launch(stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(hits.cpu().numpy().view(np.uint32), _run_multi(s, rays2, offs, seg_inst, 0))
    g.close()


def test_autotune_keeps_results(native):
    import torch

    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    w = wl.config3(12, 500, 5000, 300, 3000)
    from heavyrt_gb300 import SceneRT

    s = SceneRT()
    ids = s.add_geoms_batched(w.verts, w.idx)
    for gid in ids:
        s.AddInstance(gid)
    s.CommitScene()
    seg_inst = np.arange(len(ids), dtype=np.uint32)
    want = _run_multi(s, w.rays, w.ray_offsets, seg_inst, 0)
    dr = torch.from_numpy(w.rays).cuda()
    do = torch.from_numpy(w.ray_offsets.view(np.int32)).cuda()
    ds = torch.from_numpy(seg_inst.view(np.int32)).cuda()
    out = torch.zeros((len(w.rays), 8), dtype=torch.int32, device="cuda")
    d = E.query_desc(0, dr.data_ptr(), len(w.rays), out.data_ptr(), do.data_ptr(), ds.data_ptr(), len(ids))
    cfg, ms = s.autotune(d, repeats=1)
    assert ms > 0 and cfg == s.trace_config(0)
    assert cfg["threadsPerBlock"] in (64, 128, 256) and cfg["persistent"] in (0, 1)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), want)
    np.testing.assert_array_equal(_run_multi(s, w.rays, w.ray_offsets, seg_inst, 0), want)


def test_full_size_batch_sampled_vs_oracle(native):
    """256 soups, 12.7M triangles in one segmented build; the rays of eight
    scenes (smallest, largest and six others) checked against the oracle."""
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    w = wl.config3()
    s = SceneRT()
    ids = s.add_geoms_batched(w.verts, w.idx)
    for gid in ids:
        s.AddInstance(gid)
    s.CommitScene()
    seg_inst = np.arange(len(ids), dtype=np.uint32)
    got = _run_multi(s, w.rays, w.ray_offsets, seg_inst, 0)
    got_any = _run_multi(s, w.rays, w.ray_offsets, seg_inst, 1)
    tris = np.array(w.params["tri_counts"])
    pick = sorted({int(tris.argmin()), int(tris.argmax()), 1, 50, 100, 150, 200, 255})
    for k in pick:
        a, b = w.ray_offsets[k], w.ray_offsets[k + 1]
        o = orc.OracleBVH(w.verts[k], w.idx[k])
        want = o.trace(w.rays[a:b]).view(np.uint32).reshape(-1, 8).copy()
        hit = want[:, 1] != MISS
        want[hit, 2] = k
        want[hit, 3] = ids[k]
        np.testing.assert_array_equal(got[a:b], want)
        np.testing.assert_array_equal(got_any[a:b], o.trace(w.rays[a:b], any_hit=True))
        assert s.geom_info(ids[k])["leaves"] == o.n_leaves
