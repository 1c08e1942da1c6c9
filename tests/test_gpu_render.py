"""Frames of HeavyRT's two example renderers on the GPU (hrt_frame): every
stage equals the renderers' own kernels (fixture from the reference's
eye_ray.cpp / rtao.cpp) and the C restatement bit for bit, in every node
layout, with instances, at full HD, and with the error paths reported."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _fixture():
    return dict(np.load(GOLDEN / "render_frames.npz"))


def _case(z, k):
    w, h, r = (int(x) for x in z[f"{k}_params"])
    zn, zf, rad, pw = (float(x) for x in z[f"{k}_fparams"])
    return dict(proj_inv=z[f"{k}_proj_inv"], world_view_inv=z[f"{k}_world_view_inv"], width=w, height=h, z_near=zn,
                z_far=zf, rays_per_pixel=r, radius=rad, power=pw, norm_matrix=z[f"{k}_norm_matrix"])


def _scene(verts, idx, layout=0, instances=None):
    from heavyrt_gb300 import SceneRT

    s = SceneRT(layout=layout)
    g = s.AddGeom_Triangles3f(verts, len(verts), idx, idx.size, vByteStride=16)
    for m in instances if instances is not None else [None]:
        s.AddInstance(g, m)
    s.CommitScene()
    return s, g


def _render_rtao(frame, scene, c, colors, norm_matrices=None):
    import torch

    nm = norm_matrices if norm_matrices is not None else c["norm_matrix"][None]
    frame.render_rtao(scene, c["proj_inv"], c["world_view_inv"], c["width"], c["height"], colors.data_ptr(),
                      c["z_near"], c["z_far"], c["radius"], c["power"], nm)
    torch.cuda.synchronize()
    from heavyrt_gb300 import engine as E

    out = {"colors": colors.cpu().numpy().view(np.uint32).copy(),
           "positions": frame.read(E.FRAME_POSITIONS), "visibility": frame.read(E.FRAME_VISIBILITY),
           "ao_pixel": frame.read(E.FRAME_AO_PIXEL), "ao_rays": frame.read(E.FRAME_AO_RAYS),
           "ao_hit": frame.read(E.FRAME_AO_HITS), "ray_pixel": frame.read(E.FRAME_RAY_PIXEL),
           "eye_hits": frame.read(E.FRAME_EYE_HITS), "eye_rays": frame.read(E.FRAME_EYE_RAYS)}
    # AO rays per (pixel, sample), pixels in row-major order, as the renderer loops
    r = c["rays_per_pixel"]
    order = np.argsort(out["ao_pixel"], kind="stable")
    out["ao_rays_by_pixel"] = out["ao_rays"].reshape(-1, r, 8)[order].reshape(-1, 8)
    out["ao_hit_by_pixel"] = out["ao_hit"].reshape(-1, r)[order].reshape(-1)
    return out


def test_rtao_frame_matches_reference_fixture(native):
    """Both fixture frames: hit points with packed normals, AO rays, occlusion,
    visibility and colours equal the reference RTAO kernels bit for bit."""
    import torch

    from heavyrt_gb300 import Frame, PinnedBuffer, rtao_qmc_tile

    z = _fixture()
    s, g = _scene(z["verts"], z["idx"])
    f = Frame()
    f.set_normals(g, z["normals"])
    for k in ("a", "b"):
        c = _case(z, k)
        f.set_ao_tile(rtao_qmc_tile(c["rays_per_pixel"]), c["rays_per_pixel"])
        colors = torch.empty(c["width"] * c["height"], dtype=torch.int32, device="cuda")
        o = _render_rtao(f, s, c, colors)
        # the same frame into page-locked host memory
        pin = PinnedBuffer(4 * c["width"] * c["height"])
        f.render_rtao(s, c["proj_inv"], c["world_view_inv"], c["width"], c["height"], pin.ptr, c["z_near"],
                      c["z_far"], c["radius"], c["power"], c["norm_matrix"][None])
        np.testing.assert_array_equal(pin.array(np.uint32), z[f"{k}_colors"])
        pin.free()
        hit = z[f"{k}_positions"][:, 1] < 1e7
        np.testing.assert_array_equal(o["positions"].view(np.uint32), z[f"{k}_positions"].view(np.uint32))
        np.testing.assert_array_equal(np.sort(o["ao_pixel"]), np.nonzero(hit)[0])
        np.testing.assert_array_equal(o["ao_rays_by_pixel"].view(np.uint32), z[f"{k}_ao_rays"].view(np.uint32))
        np.testing.assert_array_equal(o["ao_hit_by_pixel"], z[f"{k}_ao_hit"])
        np.testing.assert_array_equal(o["visibility"].view(np.uint32), z[f"{k}_visibility"].view(np.uint32))
        np.testing.assert_array_equal(o["colors"], z[f"{k}_colors"])
        # the trace order: packed (kernel_PackXY) when both sides are multiples of 8
        if c["width"] % 8 == 0 and c["height"] % 8 == 0:
            packed = z[f"{k}_eye_packed"]
            np.testing.assert_array_equal(o["ray_pixel"], (packed >> 16) * c["width"] + (packed & 0xFFFF))
        else:
            np.testing.assert_array_equal(o["ray_pixel"], np.arange(c["width"] * c["height"], dtype=np.uint32))


def test_eye_frame_matches_reference_fixture(native):
    import torch

    from heavyrt_gb300 import Frame
    from oracle import oracle as orc

    z = _fixture()
    s, _ = _scene(z["verts"], z["idx"])
    f = Frame()
    c = _case(z, "a")
    colors = torch.empty(c["width"] * c["height"], dtype=torch.int32, device="cuda")
    f.render_eye(s, c["proj_inv"], c["world_view_inv"], c["width"], c["height"], colors.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(colors.cpu().numpy().view(np.uint32), z["a_eye_colors"])
    # colours into page-locked and into pageable host memory
    from heavyrt_gb300 import PinnedBuffer

    pin = PinnedBuffer(4 * c["width"] * c["height"])
    f.render_eye(s, c["proj_inv"], c["world_view_inv"], c["width"], c["height"], pin.ptr)
    np.testing.assert_array_equal(pin.array(np.uint32), z["a_eye_colors"])
    host = np.zeros(c["width"] * c["height"], np.uint32)
    f.render_eye(s, c["proj_inv"], c["world_view_inv"], c["width"], c["height"], host.ctypes.data)
    np.testing.assert_array_equal(host, z["a_eye_colors"])
    pin.free()
    # a size that is no multiple of 8 (row order) against the restatement
    b = orc.OracleBVH(z["verts"], z["idx"])
    colors = torch.empty(45 * 23, dtype=torch.int32, device="cuda")
    f.render_eye(s, c["proj_inv"], c["world_view_inv"], 45, 23, colors.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(colors.cpu().numpy().view(np.uint32),
                                  orc.eye_frame(b, c["proj_inv"], c["world_view_inv"], 45, 23))


@pytest.mark.parametrize("layout", [0, 1, 2, 3])
def test_rtao_frame_every_layout_vs_oracle(native, layout):
    """One scene, four node layouts: the frame equals the oracle's frame."""
    import torch

    from heavyrt_gb300 import Frame, rtao_qmc_tile
    from oracle import oracle as orc

    z = _fixture()
    c = _case(z, "a")
    c.update(width=96, height=72, rays_per_pixel=8, radius=0.2)
    s, g = _scene(z["verts"], z["idx"], layout)
    f = Frame()
    f.set_normals(g, z["normals"])
    f.set_ao_tile(rtao_qmc_tile(8), 8)
    colors = torch.empty(96 * 72, dtype=torch.int32, device="cuda")
    o = _render_rtao(f, s, c, colors)
    b = orc.OracleBVH(z["verts"], z["idx"])
    want = orc.rtao_frame(b, z["verts"], z["normals"], c["proj_inv"], c["world_view_inv"], 96, 72, c["z_near"],
                          c["z_far"], 8, 0.2, 1.0, c["norm_matrix"])
    np.testing.assert_array_equal(o["positions"].view(np.uint32), want["positions"].view(np.uint32))
    np.testing.assert_array_equal(o["ao_rays_by_pixel"].view(np.uint32), want["ao_rays"][want["ao_valid"]].view(np.uint32))
    np.testing.assert_array_equal(o["ao_hit_by_pixel"], want["ao_hit"][want["ao_valid"]])
    np.testing.assert_array_equal(o["colors"], want["colors"])


def test_rtao_frame_with_instances(native):
    """Two geometries under three transformed instances (two-level scene): the
    shading of each hit uses its geometry's normals and its instance's normal
    matrix; every stage after the eye query equals the restatement run on the
    GPU's eye hits, and the AO occlusion equals the engine's own any-hit query."""
    import torch

    from heavyrt_gb300 import Frame, SceneRT, rtao_qmc_tile
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    z = _fixture()
    v0, i0, n0 = z["verts"], z["idx"], z["normals"]
    v1, i1, _ = wl.heightfield(9, 20, 12)
    v1 = v1.copy()
    v1[:, :3] *= 0.4
    p1 = v1[:, :3].astype(np.float64)
    t1 = i1.reshape(-1, 3)
    fn = np.cross(p1[t1[:, 1]] - p1[t1[:, 0]], p1[t1[:, 2]] - p1[t1[:, 0]])
    n1 = np.zeros_like(p1)
    for kk in range(3):
        np.add.at(n1, t1[:, kk], fn)
    n1 = np.concatenate([n1 / np.linalg.norm(n1, axis=1, keepdims=True), np.zeros((len(n1), 1))], 1).astype(np.float32)

    def rot(a, t, sc):
        m = np.eye(4)
        m[:3, :3] = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]]) * sc
        m[:3, 3] = t
        return m.astype(np.float32)

    mats = [np.eye(4, dtype=np.float32), rot(0.4, (0.5, 0.3, 0.35), 1.0), rot(-0.9, (-0.6, 0.2, 0.3), 1.3)]
    s = SceneRT()
    g0 = s.AddGeom_Triangles3f(v0, len(v0), i0, i0.size, vByteStride=16)
    g1 = s.AddGeom_Triangles3f(v1, len(v1), i1, i1.size, vByteStride=16)
    geom_of = [g0, g1, g1]
    for gi, m in zip(geom_of, mats):
        s.AddInstance(gi, m)
    s.CommitScene()
    norm_m = np.stack([np.linalg.inv(m.astype(np.float64)).T.astype(np.float32) for m in mats])
    f = Frame()
    f.set_normals(g0, n0)
    f.set_normals(g1, n1)
    f.set_ao_tile(rtao_qmc_tile(4), 4)
    c = _case(z, "a")
    c.update(width=80, height=64, rays_per_pixel=4, radius=0.25)
    colors = torch.empty(80 * 64, dtype=torch.int32, device="cuda")
    o = _render_rtao(f, s, c, colors, norm_m)
    hits = o["eye_hits"].reshape(-1).view(orc.HIT_DTYPE)
    assert {0, 1, 2} <= set(np.unique(hits["instId"][hits["geomId"] != 0xFFFFFFFF]).tolist())
    # the restatement, from the GPU's eye rays and hits
    eye = o["eye_rays"]
    pix = o["ray_pixel"]
    sorted_idx = [s.export(g0, 7), s.export(g1, 7)]
    pos_traced = orc.rtao_positions(eye, hits, [(sorted_idx[0], v0, n0), (sorted_idx[1], v1, n1)], norm_m)
    want_pos = np.zeros_like(pos_traced)
    want_pos[pix] = pos_traced
    np.testing.assert_array_equal(o["positions"].view(np.uint32), want_pos.view(np.uint32))
    tile = rtao_qmc_tile(4)
    ao = orc.rtao_ao_rays(want_pos, 80, 64, 4, tile, 0.25)
    valid = np.repeat(want_pos[:, 1] < 1e7, 4)
    np.testing.assert_array_equal(o["ao_rays_by_pixel"].view(np.uint32), ao[valid].view(np.uint32))
    any_hit = s.RayQuery_AnyHit(ao[valid]).astype(np.uint8)
    np.testing.assert_array_equal(o["ao_hit_by_pixel"], any_hit)
    full = np.zeros(ao.shape[0], np.uint8)
    full[valid] = any_hit
    vis, col = orc.rtao_colors(want_pos, full, 4, 1.0)
    np.testing.assert_array_equal(o["colors"], col)
    assert 0 < any_hit.mean() < 1


def test_rtao_frame_full_hd_sampled(native):
    """1920x1080, 16 samples, on the 1M-vertex heightfield: colours and hit
    points of 2,000 sampled pixels equal the restatement's, and a second render
    is identical."""
    import torch

    from heavyrt_gb300 import Frame, SceneRT, rtao_qmc_tile
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    v, idx, _ = wl.heightfield(1, 1024, 1024)
    nrm = wl.vertex_normals(v, idx)
    s = SceneRT(layout=2)
    g = s.AddGeom_Triangles3f(v, len(v), idx, idx.size, vByteStride=16)
    s.AddInstance(g)
    s.CommitScene()
    f = Frame()
    f.set_normals(g, nrm)
    f.set_ao_tile(rtao_qmc_tile(16), 16)
    W, H = 1920, 1080
    p, wv = wl.camera_inverses((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, W, H)
    c = dict(proj_inv=p, world_view_inv=wv, width=W, height=H, z_near=0.0, z_far=3.4028234663852886e38,
             rays_per_pixel=16, radius=0.2, power=1.0, norm_matrix=np.eye(4, dtype=np.float32))
    colors = torch.empty(W * H, dtype=torch.int32, device="cuda")
    o = _render_rtao(f, s, c, colors)
    again = _render_rtao(f, s, c, torch.empty_like(colors))
    np.testing.assert_array_equal(o["colors"], again["colors"])
    np.testing.assert_array_equal(o["ao_hit"], again["ao_hit"])
    hit = o["positions"][:, 1] < 1e7
    assert 0.05 < hit.mean() < 0.95
    rng = np.random.default_rng(3)
    sample = np.sort(rng.choice(np.nonzero(hit)[0], 2000, replace=False))
    b = orc.OracleBVH(v, idx)
    rays = orc.eye_rays(p, wv, W, H, 0.0, 3.4028234663852886e38)[sample]
    pos_s = orc.rtao_positions(rays, b.trace(rays), [(b.sorted_indices(), v, nrm)], np.eye(4)[None])
    np.testing.assert_array_equal(pos_s.view(np.uint32), o["positions"][sample].view(np.uint32))
    pos_full = np.zeros((W * H, 4), np.float32)
    pos_full[:, 1] = 1e7
    pos_full[sample] = pos_s
    ao = orc.rtao_ao_rays(pos_full, W, H, 16, rtao_qmc_tile(16), 0.2)
    valid = np.repeat(pos_full[:, 1] < 1e7, 16)
    ao_hit = np.zeros(ao.shape[0], np.uint8)
    ao_hit[valid] = b.trace(ao[valid], any_hit=True)
    _, col = orc.rtao_colors(pos_full, ao_hit, 16, 1.0)
    np.testing.assert_array_equal(col[sample], o["colors"][sample])


def test_frame_errors(native):
    import torch

    from heavyrt_gb300 import Frame, HrtError, SceneRT, rtao_qmc_tile
    from heavyrt_gb300 import engine as E

    z = _fixture()
    c = _case(z, "a")
    colors = torch.empty(c["width"] * c["height"], dtype=torch.int32, device="cuda")
    f = Frame()
    s0 = SceneRT()
    s0.AddGeom_Triangles3f(z["verts"], len(z["verts"]), z["idx"], z["idx"].size, vByteStride=16)
    with pytest.raises(HrtError) as e:  # not committed
        f.render_eye(s0, c["proj_inv"], c["world_view_inv"], 8, 8, colors.data_ptr())
    assert e.value.status == E.HRT_ERR_STATE
    s, g = _scene(z["verts"], z["idx"])
    with pytest.raises(HrtError) as e:  # no sample tile
        _render_rtao(f, s, c, colors)
    assert e.value.status == E.HRT_ERR_STATE
    f.set_ao_tile(rtao_qmc_tile(4), 4)
    with pytest.raises(HrtError) as e:  # no normals
        _render_rtao(f, s, c, colors)
    assert e.value.status == E.HRT_ERR_STATE
    f.set_normals(g, z["normals"][:-1])
    with pytest.raises(HrtError) as e:  # normals of another vertex count
        _render_rtao(f, s, c, colors)
    assert e.value.status == E.HRT_ERR_STATE
    f.set_normals(g, z["normals"])
    assert E.lib().hrt_frame_render_eye(f._h, s._h, None, None, 4, 4, None, None) == E.HRT_ERR_INVALID_ARGUMENT
    with pytest.raises(HrtError):
        f.render_eye(s, c["proj_inv"], c["world_view_inv"], 4, 4, 0)
    with pytest.raises(HrtError):
        f.render_eye(s, c["proj_inv"], c["world_view_inv"], 70000, 1, colors.data_ptr())
    with pytest.raises(ValueError):
        f.set_ao_tile(np.zeros(10, np.float32), 4)
    # a zero-sized frame is a no-op, and the frame still renders afterwards
    f.render_eye(s, c["proj_inv"], c["world_view_inv"], 0, 0, 0)
    o = _render_rtao(f, s, c, colors)
    assert o["colors"].shape[0] == c["width"] * c["height"]
