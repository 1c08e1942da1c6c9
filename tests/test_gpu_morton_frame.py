"""The cubic Morton frame (HRT_OPTION_MORTON_FRAME = HRT_MORTON_CUBIC): the
same LBVH on a grid with one scale for all three axes.  Against the oracle
built on the same grid (oracle/hrt_oracle.c zindex_scale with cubic != 0)
every build stage and every binary-layout hit is bit-exact; against the
reference's own per-axis build the tree differs, so hits are held to the
stated tolerance (hit/miss and any-hit exact, another triangle only at a tie
within 1e-5 relative t)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF
LAYOUTS = [("bvh2", None), ("bvh4", 1), ("bvh4_f16", 1), ("bvh4_q8", 1), ("bvh4_f16", 0)]


def _scene(v, idx, layout, merge, cubic=True):
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E

    s = SceneRT(layout=layout)
    if merge is not None:
        s.set_bvh4_merge(merge)
    if cubic:
        s.set_morton_frame(E.MORTON_CUBIC)
    gid = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
    s.AddInstance(gid)
    s.CommitScene()
    return s, gid


def _u32(h):
    return np.ascontiguousarray(h).view(np.uint32).reshape(-1, 8)


def _within_tolerance(got, want):
    g, w = _u32(got), _u32(want)
    np.testing.assert_array_equal(g[:, 3] != MISS, w[:, 3] != MISS)
    same = g[:, 1] == w[:, 1]
    np.testing.assert_array_equal(g[same], w[same])
    tg = g[~same, 0].view(np.float32).astype(np.float64)
    tw = w[~same, 0].view(np.float32).astype(np.float64)
    assert np.all(np.abs(tg - tw) <= 1e-5 * np.abs(tw))
    assert np.count_nonzero(~same) <= max(2, g.shape[0] // 100000)


def _cases():
    from heavyrt_gb300 import workload as wl

    hv, hidx, _ = wl.heightfield(21, 256, 256)
    hrays = np.concatenate([wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 240, 135),
                            wl.rays_at_triangles(3, hv, hidx, 20000, jitter=0.01)])
    sv, sidx = wl.soup(22, 30000, -1.0, 1.0, 0.03)
    sv[:, 2] *= 0.1  # a flat soup: the frames differ
    srays = np.concatenate([wl.rays_at_triangles(4, sv, sidx, 20000, jitter=0.02), wl.sphere_rays(5, 5000)])
    return [("heightfield256", hv, hidx, hrays), ("flat_soup30000", sv, sidx, srays)]


def test_cubic_frame_build_and_hits_vs_oracle(native):
    from heavyrt_gb300 import engine as E
    from oracle import oracle as orc

    for name, v, idx, rays in _cases():
        oc = orc.OracleBVH(v, idx, cubic=True)
        orf = orc.OracleBVH(v, idx)
        assert oc.n_leaves != orf.n_leaves or not np.array_equal(oc.morton_sorted(), orf.morton_sorted()), name
        want_c = oc.trace(rays)
        want_ref = orf.trace(rays)
        want_any = orf.trace(rays, any_hit=True)
        np.testing.assert_array_equal(oc.trace(rays, any_hit=True), want_any)
        for layout, merge in LAYOUTS:
            s, gid = _scene(v, idx, layout, merge)
            # every build stage bit-exact against the oracle on the same grid
            np.testing.assert_array_equal(s.export(gid, E.EXPORT_SCENE_BOX).view(np.uint32),
                                          oc.scene_box().view(np.uint32))
            np.testing.assert_array_equal(s.export(gid, E.EXPORT_MORTON_UNSORTED).reshape(-1, 2), oc.morton_unsorted())
            np.testing.assert_array_equal(s.export(gid, E.EXPORT_MORTON_SORTED).reshape(-1, 2), oc.morton_sorted())
            np.testing.assert_array_equal(s.export(gid, E.EXPORT_RUN_STARTS), oc.run_starts())
            np.testing.assert_array_equal(s.export(gid, E.EXPORT_LR_NODES).view(np.uint32).reshape(-1),
                                          oc.lr_nodes().view(np.uint32).reshape(-1))
            np.testing.assert_array_equal(s.export(gid, E.EXPORT_LR_COUNTS), oc.lr_counts())
            got = s.RayQuery_NearestHit(rays)
            if layout == "bvh2":  # the reference's traversal decisions on this tree
                np.testing.assert_array_equal(_u32(got), _u32(want_c), err_msg=name)
            else:
                _within_tolerance(got, want_c)
            # against the reference's own per-axis build: the stated tolerance,
            # triangles compared by their original index (the two trees sort
            # them differently)
            g, w = _u32(got).copy(), _u32(want_ref).copy()
            hg, hw = g[:, 3] != MISS, w[:, 3] != MISS
            g[hg, 1] = s.export(gid, E.EXPORT_PRIM_INDICES)[g[hg, 1]]
            w[hw, 1] = orf.prim_indices()[w[hw, 1]]
            same = g[:, 1] == w[:, 1]
            np.testing.assert_array_equal(g[same], w[same])
            assert np.count_nonzero(~same) <= max(2, g.shape[0] // 100000), name
            np.testing.assert_array_equal(g[:, 3] != MISS, w[:, 3] != MISS)
            tg = g[~same, 0].view(np.float32).astype(np.float64)
            tw = w[~same, 0].view(np.float32).astype(np.float64)
            assert np.all(np.abs(tg - tw) <= 1e-5 * np.abs(tw)), name
            np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), want_any, err_msg=f"{name} {layout}")
            s.close()


def test_cubic_frame_batch_refit_and_default(native, tmp_path):
    """Segmented builds keep the frame per geometry (equal to single builds),
    a refit keeps the build's frame (also after a blob round trip), and the
    default frame is the reference's."""
    import torch

    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    scenes = []
    for k, n in enumerate((3000, 700, 1)):
        v, i = wl.soup(800 + k, n, off=0.03)
        v[:, 1] *= 0.2
        scenes.append((v, i))
    s = SceneRT(layout="bvh4_f16")
    s.set_bvh4_merge(1)
    s.set_morton_frame(E.MORTON_CUBIC)
    ids = s.add_geoms_batched([v for v, _ in scenes], [i for _, i in scenes])
    for gid, (v, i) in zip(ids, scenes):
        oc = orc.OracleBVH(v, i, cubic=True)
        np.testing.assert_array_equal(s.export(gid, E.EXPORT_MORTON_SORTED).reshape(-1, 2), oc.morton_sorted())
        np.testing.assert_array_equal(s.export(gid, E.EXPORT_LR_NODES).view(np.uint32).reshape(-1),
                                      oc.lr_nodes().view(np.uint32).reshape(-1))
    s.close()

    v, i = scenes[0]
    rays = wl.rays_at_triangles(9, v, i, 5000, jitter=0.02)
    moved = v.copy()
    moved[:, :3] += np.random.default_rng(3).uniform(-0.005, 0.005, (v.shape[0], 3)).astype(np.float32)
    s, gid = _scene(v, i, "bvh2", None)
    before = s.export(gid, E.EXPORT_SCENE_BOX).view(np.uint32)[8:11].copy()  # the Morton scales
    s.UpdateGeom_Triangles3f(gid, moved, moved.shape[0], i, i.size, E.BUILD_REFIT, 16)
    s.CommitScene()
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_SCENE_BOX).view(np.uint32)[8:11], before)
    fresh = orc.OracleBVH(moved, i, cubic=True)
    got = _u32(s.RayQuery_NearestHit(rays))
    want = _u32(fresh.trace(rays))
    # a fresh build of the moved mesh is another tree: the same t up to the stated tie tolerance
    np.testing.assert_array_equal(got[:, 3] != MISS, want[:, 3] != MISS)
    tg, tw = got[:, 0].view(np.float32).astype(np.float64), want[:, 0].view(np.float32).astype(np.float64)
    assert np.all(np.abs(tg - tw) <= 1e-5 * np.abs(tw))
    assert np.count_nonzero(got[:, 0] != want[:, 0]) <= 2
    np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), fresh.trace(rays, any_hit=True))
    # a geometry restored from a blob refits on the grid it was built on
    blob = tmp_path / "cubic.blob"
    s.save_geom(gid, blob)
    r = SceneRT()
    gid2 = r.load_geom(blob)
    for sc, g in ((s, gid), (r, gid2)):
        sc.UpdateGeom_Triangles3f(g, v, v.shape[0], i, i.size, E.BUILD_REFIT, 16)
    np.testing.assert_array_equal(r.export(gid2, E.EXPORT_SCENE_BOX), s.export(gid, E.EXPORT_SCENE_BOX))
    np.testing.assert_array_equal(r.export(gid2, E.EXPORT_SCENE_BOX).view(np.uint32)[8:11], before)
    r.close()
    s.close()

    d = SceneRT()
    gid = d.AddGeom_Triangles3f(v, v.shape[0], i, i.size, vByteStride=16)
    np.testing.assert_array_equal(d.export(gid, E.EXPORT_MORTON_SORTED).reshape(-1, 2),
                                  orc.OracleBVH(v, i).morton_sorted())
    d.close()
