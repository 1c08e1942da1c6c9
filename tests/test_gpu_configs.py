"""The benchmark configurations in full against the oracle (the C restatement
of HeavyRT's LBVHBuilder and BVH2TraverseC32 + Moller-Trumbore,
core/builders/lbvh.cpp, core/BVH2CommonRT.cpp:9-141), through the C ABI:

  C0  65,536-triangle soup, 512 x 512 eye rays: every build stage and every
      nearest / any hit, in all four layouts;
  C1  the 2,097,152-triangle heightfield frame: all 2,073,600 eye rays
      (nearest) and all ~4M AO rays (any) of the frame, in all four layouts;
  C2  each scene separately, 2,073,600 eye rays + ~33M AO rays: the
      8,388,608-triangle soup (sorted positions up to 2^23 - 1, the upper
      half of the 24-bit leaf-start field of core/raytrace_common.h:38-51)
      with every build stage, and the heightfield seen from above, in all
      four layouts;
  C3  all 256 scenes of the segmented batch, every ray, nearest and any, in
      the binary layout and in the batched benchmark's BVH4 FP16 structure.

Integer results are bit-exact.  The binary layout makes the reference's
decisions, so its hits equal the oracle's bit for bit.  The 4-wide layouts
visit children in another order: hit/miss is exact, any-hit flags are exact,
and a different triangle is allowed only at a tie within 1e-5 relative t
(see _compare_nearest)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF
LAYOUTS = [("bvh2", None), ("bvh4", 1), ("bvh4_f16", 1), ("bvh4_q8", 1)]


def _scene(v, idx, layout, merge):
    from heavyrt_gb300 import SceneRT

    s = SceneRT(layout=layout)
    if merge is not None:
        s.set_bvh4_merge(merge)
    gid = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
    s.AddInstance(gid)
    s.CommitScene()
    return s, gid


def _trace_device(s, kind, rays):
    """One query of device-resident rays (the benchmark's path)."""
    import torch

    d = torch.from_numpy(np.ascontiguousarray(rays, dtype=np.float32)).cuda()
    n = d.shape[0]
    out = torch.empty((n, 8) if kind == 0 else (n,), dtype=torch.int32 if kind == 0 else torch.uint8, device="cuda")
    s.query_device(kind, d.data_ptr(), n, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    return got.view(np.uint32).reshape(-1, 8) if kind == 0 else got.astype(bool)


def _compare_nearest(got, want, layout):
    """got: uint32 [n, 8] hit records; want: the oracle's hits.  Returns the
    number of near ties resolved to another triangle.

    The binary layout is bit-exact.  A 4-wide layout visits children in
    another order, and its quantised boxes are larger: it may test a triangle
    that the reference's order pruned, and the reference's 1e-6 barycentric
    slack accepts hit points slightly outside a triangle's box, so such a
    triangle can give a t one rounding below the reference's.  There the
    tolerance is the stated one: the same triangle gives the same record bit
    for bit, another triangle only at a tie within 1e-5 relative t."""
    w = np.ascontiguousarray(want).view(np.uint32).reshape(-1, 8)
    if layout == "bvh2":
        np.testing.assert_array_equal(got, w)
        return 0
    np.testing.assert_array_equal(got[:, 3] != MISS, w[:, 3] != MISS)
    same = got[:, 1] == w[:, 1]
    np.testing.assert_array_equal(got[same], w[same])
    tg = got[~same, 0].view(np.float32).astype(np.float64)
    tw = w[~same, 0].view(np.float32).astype(np.float64)
    assert np.all(np.abs(tg - tw) <= 1e-5 * np.abs(tw)), (tg, tw)
    ties = int(np.count_nonzero(~same))
    assert ties <= max(2, got.shape[0] // 100000), ties
    return ties


def _check_build(s, gid, o):
    from heavyrt_gb300 import engine as E

    np.testing.assert_array_equal(s.export(gid, E.EXPORT_SCENE_BOX).view(np.uint32), o.scene_box().view(np.uint32))
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_MORTON_UNSORTED).reshape(-1, 2), o.morton_unsorted())
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_MORTON_SORTED).reshape(-1, 2), o.morton_sorted())
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_COMPRESSED), o.compressed())
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_RUN_STARTS), o.run_starts())
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_LR_NODES).view(np.uint32).reshape(-1),
                                  o.lr_nodes().view(np.uint32).reshape(-1))
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_LR_COUNTS), o.lr_counts())
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_PRIM_INDICES), o.prim_indices())
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_SORTED_INDICES), o.sorted_indices())


def _frame_vs_oracle(w, o, want_eye, ao, want_ao, check_build=False):
    """Every layout traces the frame's eye rays (nearest) and AO rays (any);
    all results against the oracle's."""
    from heavyrt_gb300 import engine as E

    checked = 0
    for layout, merge in LAYOUTS:
        s, gid = _scene(w.verts, w.idx, layout, merge)
        if check_build:
            _check_build(s, gid, o)
        np.testing.assert_array_equal(s.export(gid, E.EXPORT_PRIM_INDICES), o.prim_indices())
        _compare_nearest(_trace_device(s, 0, w.eye_rays), want_eye, layout)
        np.testing.assert_array_equal(_trace_device(s, 1, ao), want_ao, err_msg=layout)
        # the host-pointer path of the same rays
        np.testing.assert_array_equal(s.RayQuery_AnyHit(ao), want_ao, err_msg=layout)
        checked += w.eye_rays.shape[0] + ao.shape[0]
        s.close()
    return checked


def test_config0_every_stage_and_ray(native):
    """C0: 65,536-triangle soup, 512 x 512 eye rays, every build stage, every
    ray (nearest, and any-hit on the eye rays and on AO rays of the hits)."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    w = wl.config0()
    o = orc.OracleBVH(w.verts, w.idx)
    want = o.trace(w.eye_rays)
    assert (want["geomId"] != MISS).mean() > 0.3
    w.params.update({"ao_per_hit": 4, "ao_length": 0.2, "ao_offset": 1e-4, "ao_seed": wl.SEED_AO})
    ao = wl.frame_ao_rays(w, want, o.sorted_indices())
    want_ao = o.trace(ao, any_hit=True)
    assert 0 < want_ao.mean() < 1
    _frame_vs_oracle(w, o, want, ao, want_ao, check_build=True)
    s, _ = _scene(w.verts, w.idx, "bvh2", None)
    np.testing.assert_array_equal(s.RayQuery_AnyHit(w.eye_rays), o.trace(w.eye_rays, any_hit=True))
    np.testing.assert_array_equal(s.RayQuery_NearestHit(w.eye_rays).view(np.uint32).reshape(-1, 8),
                                  want.view(np.uint32).reshape(-1, 8))
    s.close()


def test_config1_full_frame_every_layout(native):
    """C1: the headline frame, all 2,073,600 eye rays and all AO rays."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    w = wl.config1()
    o = orc.OracleBVH(w.verts, w.idx)
    want = o.trace(w.eye_rays)
    ao = wl.frame_ao_rays(w, want, o.sorted_indices())
    assert ao.shape[0] > 3_900_000
    want_ao = o.trace(ao, any_hit=True)
    checked = _frame_vs_oracle(w, o, want, ao, want_ao, check_build=True)
    assert checked == 4 * (2_073_600 + ao.shape[0])


@pytest.mark.parametrize("scene", ["soup", "heightfield"])
def test_config2_each_scene_every_layout(native, scene):
    """C2, each scene separately: 2,073,600 eye rays + 16 AO rays per hit
    (~33M), every layout against the oracle; the soup's 8,388,608 triangles
    with every build stage."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    w = wl.config2(scene)
    o = orc.OracleBVH(w.verts, w.idx)
    assert o.status == 0
    want = o.trace(w.eye_rays)
    assert (want["geomId"] != MISS).mean() > 0.97
    ao = wl.frame_ao_rays(w, want, o.sorted_indices())
    assert ao.shape[0] > 32_000_000
    want_ao = o.trace(ao, any_hit=True)
    _frame_vs_oracle(w, o, want, ao, want_ao, check_build=(scene == "soup"))
    if scene == "soup":
        # hits reach the top of the sorted order (leaf starts above 2^22)
        assert int(want["primId"][want["geomId"] != MISS].max()) >= 8_000_000


def _run_multi(s, rays, offs, seg_inst, kind):
    import torch

    from heavyrt_gb300 import engine as E

    dr = torch.from_numpy(rays).cuda()
    do = torch.from_numpy(offs.view(np.int32)).cuda()
    ds = torch.from_numpy(seg_inst.view(np.int32)).cuda()
    n = len(rays)
    out = torch.zeros((n, 8) if kind == 0 else (n,), dtype=torch.int32 if kind == 0 else torch.uint8, device="cuda")
    s.query_multi(E.query_desc(kind, dr.data_ptr(), n, out.data_ptr(), do.data_ptr(), ds.data_ptr(), len(seg_inst)))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    return got.view(np.uint32).reshape(-1, 8) if kind == 0 else got.astype(bool)


def test_config3_all_256_scenes(native):
    """C3: the 256 soups built in one segmented build, every ray of every
    scene traced by one segmented launch per kind, in the binary layout and in
    the batched benchmark's structure (BVH4 FP16, merge bound 1), against one
    oracle build per scene."""
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    w = wl.config3()
    want, want_any = [], []
    for k in range(len(w.verts)):
        a, b = w.ray_offsets[k], w.ray_offsets[k + 1]
        o = orc.OracleBVH(w.verts[k], w.idx[k])
        want.append(o.trace(w.rays[a:b]).view(np.uint32).reshape(-1, 8).copy())
        want_any.append(o.trace(w.rays[a:b], any_hit=True))
        o.close()
    for layout, merge in (("bvh2", None), ("bvh4_f16", 1)):
        s = SceneRT(layout=layout)
        if merge is not None:
            s.set_bvh4_merge(merge)
        ids = s.add_geoms_batched(w.verts, w.idx)
        for gid in ids:
            s.AddInstance(gid)
        s.CommitScene()
        seg_inst = np.arange(len(ids), dtype=np.uint32)
        got = _run_multi(s, w.rays, w.ray_offsets, seg_inst, 0)
        got_any = _run_multi(s, w.rays, w.ray_offsets, seg_inst, 1)
        for k in range(len(ids)):
            a, b = w.ray_offsets[k], w.ray_offsets[k + 1]
            wk = want[k].copy()
            hit = wk[:, 1] != MISS
            wk[hit, 2] = k
            wk[hit, 3] = ids[k]
            _compare_nearest(got[a:b], wk, layout)
            np.testing.assert_array_equal(got_any[a:b], want_any[k], err_msg=f"{layout} scene {k}")
        s.close()


def test_config1_full_frame_headline_tree(native):
    """C1 on the benchmark's tree (cubic Morton grid, largest-first collapse,
    FP16 nodes, leaf merge 1): every eye ray (nearest) and every AO ray (any)
    against the oracle's reference tree.  The trees sort the triangles
    differently, so hits are compared by original triangle index: hit/miss
    and any-hit exact, another triangle only at a tie within 1e-5 relative t."""
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    w = wl.config1()
    o = orc.OracleBVH(w.verts, w.idx)
    want = o.trace(w.eye_rays)
    ao = wl.frame_ao_rays(w, want, o.sorted_indices())
    want_any = o.trace(ao, any_hit=True)
    for layout in ("bvh4_f16", "bvh4"):
        s = SceneRT(layout=layout)
        s.set_bvh4_merge(1)
        s.set_morton_frame(E.MORTON_CUBIC)
        s.set_bvh4_collapse(E.BVH4_COLLAPSE_LARGEST_FIRST)
        gid = s.AddGeom_Triangles3f(w.verts, w.verts.shape[0], w.idx, w.idx.size, vByteStride=16)
        s.AddInstance(gid)
        s.CommitScene()
        g = _trace_device(s, 0, w.eye_rays).copy()
        wv = np.ascontiguousarray(want).view(np.uint32).reshape(-1, 8).copy()
        hg, hw = g[:, 3] != MISS, wv[:, 3] != MISS
        np.testing.assert_array_equal(hg, hw, err_msg=layout)
        g[hg, 1] = s.export(gid, E.EXPORT_PRIM_INDICES)[g[hg, 1]]
        wv[hw, 1] = o.prim_indices()[wv[hw, 1]]
        same = g[:, 1] == wv[:, 1]
        np.testing.assert_array_equal(g[same], wv[same], err_msg=layout)
        tg = g[~same, 0].view(np.float32).astype(np.float64)
        tw = wv[~same, 0].view(np.float32).astype(np.float64)
        assert np.all(np.abs(tg - tw) <= 1e-5 * np.abs(tw)), layout
        assert np.count_nonzero(~same) <= max(2, g.shape[0] // 100000), layout
        np.testing.assert_array_equal(_trace_device(s, 1, ao), want_any, err_msg=layout)
        s.close()
