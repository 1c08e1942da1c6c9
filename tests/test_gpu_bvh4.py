"""4-wide layouts (FP32, FP16 and 8-bit boxes) against the oracle's binary
traversal: any-hit exact; nearest hit/miss exact, t exact, and the same
triangle except where two triangles tie in t; quantised boxes contain the FP32
boxes they stand for."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF
LAYOUTS = [1, 2, 3]  # BVH4_F32, BVH4_F16, BVH4_Q8


def _scene(v, idx, layout, merge=0):
    from heavyrt_gb300 import SceneRT

    s = SceneRT(layout=layout)
    if merge:
        s.set_bvh4_merge(merge)
    gid = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
    s.AddInstance(gid)
    s.CommitScene()
    return s, gid


def _check_nearest(got, want, sorted_idx, verts):
    found = want["geomId"] != MISS
    np.testing.assert_array_equal(got["geomId"] != MISS, found)
    np.testing.assert_array_equal(got["t"].view(np.uint32), want["t"].view(np.uint32))
    same = got["primId"] == want["primId"]
    # a different triangle is only allowed where it gives the same t (a tie)
    diff = found & ~same
    assert diff.sum() <= max(2, found.sum() // 1000)
    np.testing.assert_array_equal(got["coords"][same & found].view(np.uint32), want["coords"][same & found].view(np.uint32))


def _cases():
    from heavyrt_gb300 import workload as wl

    out = []
    for n in (1, 2, 3, 5, 300, 20000):
        v, idx = wl.soup(4000 + n, n, off=0.05)
        rays = np.concatenate([wl.rays_at_triangles(n, v, idx, 3000, jitter=0.03), wl.sphere_rays(n, 500)])
        out.append((f"soup{n}", v, idx, rays))
    v, idx, _ = wl.heightfield(99, 160, 160)
    rays = np.concatenate([wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 160, 90),
                           wl.rays_at_triangles(2, v, idx, 5000, jitter=0.01)])
    rays[::3, 3] = 1.0
    out.append(("heightfield160", v, idx, rays))
    return out


@pytest.mark.parametrize("layout,merge", [(1, 0), (2, 0), (3, 0), (1, 1), (2, 4), (3, 8)])
def test_bvh4_layouts_match_oracle(native, layout, merge):
    from heavyrt_gb300 import engine as E
    from oracle import oracle as orc

    for name, v, idx, rays in _cases():
        o = orc.OracleBVH(v, idx)
        s, gid = _scene(v, idx, layout, merge)
        for persistent in (0, 1):
            s.set_trace_config(1, persistent=persistent)
            np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), o.trace(rays, any_hit=True), err_msg=name)
        _check_nearest(s.RayQuery_NearestHit(rays), o.trace(rays), o.sorted_indices(), v)
        # the 4-wide tree shares the binary tree's sorted order
        np.testing.assert_array_equal(s.export(gid, E.EXPORT_PRIM_INDICES), o.prim_indices())
        s.close()


def _decode_f32(raw):
    n = raw.reshape(-1, 32)
    f = n[:, :24].view(np.float32).reshape(-1, 6, 4)  # lox, loy, loz, hix, hiy, hiz x 4 slots
    lo = np.stack([f[:, 0], f[:, 1], f[:, 2]], axis=2)  # [node, slot, axis]
    hi = np.stack([f[:, 3], f[:, 4], f[:, 5]], axis=2)
    return lo, hi, n[:, 24:28]


def _decode_f16(raw):
    n = raw.reshape(-1, 16)
    h = n[:, :12].copy().view(np.float16).astype(np.float32).reshape(-1, 3, 4, 2)  # word group, slot, half
    lo = np.stack([h[:, 0, :, 0], h[:, 0, :, 1], h[:, 1, :, 0]], axis=2)
    hi = np.stack([h[:, 1, :, 1], h[:, 2, :, 0], h[:, 2, :, 1]], axis=2)
    return lo, hi, n[:, 12:16]


def _decode_q8(raw):
    n = raw.reshape(-1, 16)
    org = n[:, 0:3].view(np.float32)
    e = n[:, 3]
    ex = np.stack([(e & 0xFF), (e >> 8) & 0xFF, (e >> 16) & 0xFF], axis=1).astype(np.int32) - 128
    scale = np.ldexp(np.float32(1.0), ex).astype(np.float32)
    words = n[:, 4:10]  # lo.x lo.y lo.z hi.x hi.y hi.z (4 bytes = 4 slots each)
    q = np.stack([(words >> (8 * k)) & 0xFF for k in range(4)], axis=2).astype(np.float32)  # [node, bound, slot]
    lo = np.empty((n.shape[0], 4, 3), np.float32)
    hi = np.empty((n.shape[0], 4, 3), np.float32)
    for c in range(3):
        lo[:, :, c] = org[:, c, None] + q[:, c, :] * scale[:, c, None]
        hi[:, :, c] = org[:, c, None] + q[:, 3 + c, :] * scale[:, c, None]
    return lo, hi, n[:, 12:16]


@pytest.mark.parametrize("layout", [2, 3])
def test_quantised_boxes_contain_fp32_boxes(native, layout):
    """Node numbering and refs are identical across 4-wide formats; every
    quantised slot box contains the FP32 slot box (outward rounding)."""
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(7, 200, 200)
    v2, idx2 = wl.soup(8, 30000, off=0.005)
    for vv, ii in ((v, idx), (v2, idx2)):
        s32, g32 = _scene(vv, ii, 1)
        sq, gq = _scene(vv, ii, layout)
        lo32, hi32, ref32 = _decode_f32(s32.export(g32, E.EXPORT_NODES4))
        loq, hiq, refq = (_decode_f16 if layout == 2 else _decode_q8)(sq.export(gq, E.EXPORT_NODES4))
        np.testing.assert_array_equal(ref32, refq)
        used = ref32 != MISS
        assert np.all(loq[used] <= lo32[used]) and np.all(hiq[used] >= hi32[used])
        # and not grossly larger than the frame allows
        ext = (hi32[used] - lo32[used]).max()
        assert np.all(hiq[used] - loq[used] <= (hi32[used] - lo32[used]) + 2 * max(ext, 1e-3))


def test_bvh4_fetches_fewer_nodes(native):
    import torch

    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(5, 256, 256)
    rays = np.concatenate([wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 128, 72),
                           wl.rays_at_triangles(4, v, idx, 5000, jitter=0.01)])
    dr = torch.from_numpy(rays).cuda()
    counts = {}
    for layout in (0, 1, 2, 3):
        s, _ = _scene(v, idx, layout)
        counts[layout] = s.query_counters(0, dr.data_ptr(), rays.shape[0])
        s.close()
    assert counts[1][0] < counts[0][0]
    # quantised boxes only add visits
    assert counts[2][0] >= counts[1][0] and counts[3][0] >= counts[1][0]


def test_layout_after_geometry_is_rejected(native):
    from heavyrt_gb300 import HrtError, SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    s = SceneRT()
    v, idx = wl.soup(1, 10)
    s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
    with pytest.raises(HrtError) as e:
        s.ctx.check(E.lib().hrt_scene_set_layout(s._h, 1), "layout")
    assert e.value.status == E.HRT_ERR_STATE
    assert SceneRT(layout="bvh4_q8").layout == E.LAYOUT_BVH4_Q8
