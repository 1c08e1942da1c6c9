"""Ray generation on the GPU: the renderers' eye rays equal the reference's
set-up bit for bit, the benchmark camera and AO rays equal the host
generator's bit for bit, and a frame chained on the device gives the
host-chained frame's results."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _eye_cases():
    z = np.load(GOLDEN / "raygen_eye.npz")
    k = 0
    while f"rays{k}" in z:
        yield (z[f"proj_inv{k}"], z[f"world_view_inv{k}"], *[int(x) for x in z[f"size{k}"]],
               *[float(x) for x in z[f"range{k}"]], z[f"rays{k}"])
        k += 1


def test_renderer_eye_rays_bit_exact(native):
    import torch

    from heavyrt_gb300 import Context
    from oracle import oracle as orc

    ctx = Context(0)
    for p, v, w, h, tn, tf, want in _eye_cases():
        out = torch.empty((w * h, 8), dtype=torch.float32, device="cuda")
        ctx.gen_eye_rays(p, v, w, h, tn, tf, out.data_ptr())
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
        np.testing.assert_array_equal(got.view(np.uint32), orc.eye_rays(p, v, w, h, tn, tf).view(np.uint32))
    # full HD on the heightfield camera against the restatement
    p, v = next(_eye_cases())[:2]
    out = torch.empty((1920 * 1080, 8), dtype=torch.float32, device="cuda")
    ctx.gen_eye_rays(p, v, 1920, 1080, 0.0, 1e9, out.data_ptr())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32),
                                  orc.eye_rays(p, v, 1920, 1080, 0.0, 1e9).view(np.uint32))


@pytest.mark.parametrize("cam", [((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 1920, 1080),
                                 ((0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0, 512, 512),
                                 ((1.5, 2.0, -0.7), (0.1, -0.2, 0.3), (0, 1, 0), 35.0, 97, 13)])
def test_pinhole_rays_equal_host_generator(native, cam):
    import torch

    from heavyrt_gb300 import Context
    from heavyrt_gb300 import workload as wl

    eye, target, up, fov, w, h = cam
    ctx = Context(0)
    out = torch.empty((w * h, 8), dtype=torch.float32, device="cuda")
    ctx.gen_pinhole_rays(eye, target, up, fov, w, h, 0.0, 1e9, out.data_ptr())
    torch.cuda.synchronize()
    want = wl.camera_rays(eye, target, up, fov, w, h, 0.0, 1e9)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), want.view(np.uint32))


def _frame(nx=256, width=480, height=270):
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import workload as wl

    w = wl.config1(nx, width, height)
    s = SceneRT()
    g = s.AddGeom_Triangles3f(w.verts, len(w.verts), w.idx, w.idx.size, vByteStride=16)
    s.AddInstance(g)
    s.CommitScene()
    return w, s, g


def test_ao_rays_match_host_generator(native):
    import torch

    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    w, s, g = _frame()
    p = w.params
    hits = s.RayQuery_NearestHit(w.eye_rays)
    want, want_owner = wl.ao_rays(p["ao_seed"], w.eye_rays, hits, w.verts, s.export(g, E.EXPORT_SORTED_INDICES),
                                  p["ao_per_hit"], p["ao_length"], p["ao_offset"])
    d_eye = torch.from_numpy(w.eye_rays).cuda()
    d_hits = torch.from_numpy(hits.view(np.float32).reshape(-1, 8).copy()).cuda()
    cap = len(w.eye_rays) * p["ao_per_hit"]
    d_ao = torch.empty((cap, 8), dtype=torch.float32, device="cuda")
    d_owner = torch.empty(cap, dtype=torch.int32, device="cuda")
    n = s.gen_ao_rays(p["ao_seed"], d_eye.data_ptr(), d_hits.data_ptr(), len(w.eye_rays), p["ao_per_hit"],
                      p["ao_length"], p["ao_offset"], d_ao.data_ptr(), cap, d_owner.data_ptr())
    assert n == len(want) > 1000
    got = d_ao[:n].cpu().numpy()
    np.testing.assert_array_equal(d_owner[:n].cpu().numpy().view(np.uint32), want_owner)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    # too small an output buffer is reported, not overrun
    with pytest.raises(E.HrtError) as ei:
        s.gen_ao_rays(p["ao_seed"], d_eye.data_ptr(), d_hits.data_ptr(), len(w.eye_rays), p["ao_per_hit"],
                      p["ao_length"], p["ao_offset"], d_ao.data_ptr(), n - 1)
    assert ei.value.status == E.HRT_ERR_CAPACITY


def test_frame_chained_on_device(native):
    """Pinhole rays -> nearest -> AO rays -> any, all on the device, against
    the host-generated frame traced by the oracle."""
    import torch

    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    w, s, g = _frame(128, 320, 180)
    p = w.params
    ctx = s.ctx
    n_eye = len(w.eye_rays)
    d_eye = torch.empty((n_eye, 8), dtype=torch.float32, device="cuda")
    ctx.gen_pinhole_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 320, 180, 0.0, 1e9, d_eye.data_ptr())
    d_hits = torch.empty((n_eye, 8), dtype=torch.int32, device="cuda")
    s.query_device(0, d_eye.data_ptr(), n_eye, d_hits.data_ptr())
    cap = n_eye * p["ao_per_hit"]
    d_ao = torch.empty((cap, 8), dtype=torch.float32, device="cuda")
    n = s.gen_ao_rays(p["ao_seed"], d_eye.data_ptr(), d_hits.data_ptr(), n_eye, p["ao_per_hit"], p["ao_length"],
                      p["ao_offset"], d_ao.data_ptr(), cap)
    d_any = torch.empty(n, dtype=torch.uint8, device="cuda")
    s.query_device(1, d_ao.data_ptr(), n, d_any.data_ptr())
    torch.cuda.synchronize()
    o = orc.OracleBVH(w.verts, w.idx)
    hits = o.trace(w.eye_rays)
    np.testing.assert_array_equal(d_hits.cpu().numpy().view(np.uint32), hits.view(np.uint32).reshape(-1, 8))
    ao, _ = wl.ao_rays(p["ao_seed"], w.eye_rays, hits, w.verts, o.sorted_indices(), p["ao_per_hit"], p["ao_length"],
                       p["ao_offset"])
    assert len(ao) == n
    np.testing.assert_array_equal(d_ao[:n].cpu().numpy().view(np.uint32), ao.view(np.uint32))
    np.testing.assert_array_equal(d_any.cpu().numpy().astype(bool), o.trace(ao, any_hit=True))
