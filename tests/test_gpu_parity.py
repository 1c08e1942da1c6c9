"""GPU engine vs the oracle / golden vectors: every build stage and every
query result bit-exact (integer and float), through the C ABI."""
import numpy as np
import pytest

from conftest import GOLDEN, golden_cases

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF


def _load(case):
    return dict(np.load(GOLDEN / f"golden_{case}.npz"))


def _scene(verts, idx, stride=16, instances=None):
    from heavyrt_gb300 import SceneRT

    s = SceneRT()
    v = np.ascontiguousarray(verts, dtype=np.float32)
    if stride != 16:
        v3 = v.reshape(-1, 4)[:, :3]
        pad = stride // 4 - 3
        v = np.ascontiguousarray(np.concatenate([v3, np.full((v3.shape[0], pad), 7.0, np.float32)], axis=1)) if pad else \
            np.ascontiguousarray(v3)
    gid = s.AddGeom_Triangles3f(v, v.size * 4 // stride, idx, idx.size, vByteStride=stride)
    if instances is None:
        s.AddInstance(gid, np.eye(4, dtype=np.float32))
    else:
        for m in instances:
            s.AddInstance(gid, m)
    s.CommitScene()
    return s, gid


def _check_build(s, gid, want):
    from heavyrt_gb300 import engine as E

    np.testing.assert_array_equal(s.export(gid, E.EXPORT_SCENE_BOX).view(np.uint32), want["scene_box"].view(np.uint32))
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_MORTON_UNSORTED).reshape(-1, 2), want["morton_unsorted"])
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_MORTON_SORTED).reshape(-1, 2), want["morton_sorted"])
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_COMPRESSED), want["compressed"])
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_RUN_STARTS), want["run_starts"])
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_LR_NODES).view(np.uint32).reshape(-1),
                                  np.asarray(want["lr_nodes"]).view(np.uint32).reshape(-1))
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_LR_COUNTS), want["lr_counts"])
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_PRIM_INDICES), want["prim_indices"])
    np.testing.assert_array_equal(s.export(gid, E.EXPORT_SORTED_INDICES), want["sorted_indices"])


@pytest.mark.parametrize("case", golden_cases())
def test_golden_build_and_queries(native, case):
    g = _load(case)
    s, gid = _scene(g["verts"], g["idx"])
    _check_build(s, gid, g)
    hits = s.RayQuery_NearestHit(g["rays"])
    np.testing.assert_array_equal(hits.view(np.uint32).reshape(-1, 8), g["hits"].reshape(-1, 8))
    np.testing.assert_array_equal(s.RayQuery_AnyHit(g["rays"]), g["any"])


def _oracle_expect(verts, idx):
    from oracle import oracle as orc

    o = orc.OracleBVH(verts, idx)
    return o, {"scene_box": o.scene_box(), "morton_unsorted": o.morton_unsorted(), "morton_sorted": o.morton_sorted(),
               "compressed": o.compressed(), "run_starts": o.run_starts(), "lr_nodes": o.lr_nodes(),
               "lr_counts": o.lr_counts(), "prim_indices": o.prim_indices(), "sorted_indices": o.sorted_indices()}


SIZES = [1, 2, 3, 17, 255, 256, 257, 4095, 4096, 4097, 70001]


@pytest.mark.parametrize("n", SIZES)
def test_soup_sizes_vs_oracle(native, n):
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(900 + n, n, off=0.05)
    rays = np.concatenate([wl.rays_at_triangles(n, v, idx, 3000, jitter=0.03), wl.sphere_rays(n, 1000)])
    o, want = _oracle_expect(v, idx)
    s, gid = _scene(v, idx)
    _check_build(s, gid, want)
    np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32), o.trace(rays).view(np.uint32))
    np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), o.trace(rays, any_hit=True))


@pytest.mark.parametrize("stride", [12, 16, 20, 32])
def test_vertex_strides(native, stride):
    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(40 + stride, 40, 30)
    rays = wl.rays_at_triangles(stride, v, idx, 2000, jitter=0.02)
    o, want = _oracle_expect(v, idx)
    s, gid = _scene(v, idx, stride=stride)
    _check_build(s, gid, want)
    np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32), o.trace(rays).view(np.uint32))


def test_heightfield_runs_and_tnear(native):
    """Multi-triangle leaves (equal Morton codes), tNear > 0, short tFar."""
    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(77, 200, 200)
    rays = np.concatenate([wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 160, 90),
                           wl.rays_at_triangles(1, v, idx, 5000, jitter=0.01)])
    rays[::2, 3] = 2.0
    rays[1::4, 7] = 2.7
    o, want = _oracle_expect(v, idx)
    assert o.n_leaves < o.n_tris  # runs of equal codes are present
    s, gid = _scene(v, idx)
    _check_build(s, gid, want)
    np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32), o.trace(rays).view(np.uint32))
    np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), o.trace(rays, any_hit=True))


def test_counters_match_oracle(native):
    """Node-pair fetches and triangle tests per batch equal the oracle's: the
    traversal visits exactly the reference's nodes in the reference's order."""
    import torch

    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(8, 128, 128)
    rays = np.concatenate([wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 128, 72),
                           wl.sphere_rays(3, 2000)])
    o, _ = _oracle_expect(v, idx)
    s, _ = _scene(v, idx)
    dr = torch.from_numpy(rays).cuda()
    _, ocnt, _ = o.trace(rays, counters=True)
    assert s.query_counters(0, dr.data_ptr(), rays.shape[0]) == ocnt
    # any-hit: the reference finishes the leaf before leaving the loop
    # (core/BVH2CommonRTStacklessLBVH.cpp:65); the engine returns at the first
    # accepted triangle, so it visits the same node pairs and tests at most as
    # many triangles.
    _, ocnt, _ = o.trace(rays, any_hit=True, counters=True)
    gpairs, gtris = s.query_counters(1, dr.data_ptr(), rays.shape[0])
    assert gpairs == ocnt[0] and gtris <= ocnt[1]


CONFIGS = [(64, 0, 1, 1), (128, 0, 1, 1), (256, 0, 1, 1), (128, 1, 1, 1), (128, 1, 4, 16), (256, 1, 32, 32),
           (64, 1, 2, 8), (128, 1, 16, 24)]


@pytest.mark.parametrize("cfg", CONFIGS)
def test_trace_configs_give_identical_results(native, cfg):
    """The launch shape (block size, persistent pool, refill policy) never
    changes a result."""
    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(21, 96, 96)
    rays = np.concatenate([wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 96, 54),
                           wl.rays_at_triangles(3, v, idx, 6000, jitter=0.02)])
    o, _ = _oracle_expect(v, idx)
    s, _ = _scene(v, idx)
    for kind in (0, 1):
        s.set_trace_config(kind, *cfg)
        assert tuple(s.trace_config(kind).values())[:len(cfg)] == tuple(cfg)
    np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32), o.trace(rays).view(np.uint32))
    np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), o.trace(rays, any_hit=True))


def test_device_queries_match_host_queries(native):
    import torch

    from heavyrt_gb300 import HIT_DTYPE
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(5, 20000)
    rays = wl.rays_at_triangles(9, v, idx, 10000, jitter=0.02)
    s, _ = _scene(v, idx)
    dr = torch.from_numpy(rays).cuda()
    dh = torch.empty((rays.shape[0], 8), dtype=torch.int32, device="cuda")
    da = torch.empty(rays.shape[0], dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    s.query_device(0, dr.data_ptr(), rays.shape[0], dh.data_ptr(), stream)
    s.query_device(1, dr.data_ptr(), rays.shape[0], da.data_ptr(), stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dh.cpu().numpy().view(np.uint32), s.RayQuery_NearestHit(rays).view(np.uint32).reshape(-1, 8))
    np.testing.assert_array_equal(da.cpu().numpy().astype(bool), s.RayQuery_AnyHit(rays))
    assert HIT_DTYPE.itemsize == 32


def test_large_host_queries_are_pipelined_exactly(native):
    """Host-pointer queries of more than 2^18 rays run as overlapped chunks on
    three streams, and page-locked arrays are read (and any-hit flags written)
    in place; the results equal one device query of the whole batch, for an
    uneven last chunk, from pageable and from page-locked host memory."""
    import torch

    from heavyrt_gb300 import PinnedBuffer
    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(3, 200, 200)
    rays = np.concatenate([wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 700, 500),
                           wl.rays_at_triangles(4, v, idx, 300001, jitter=0.02)])
    n = rays.shape[0]
    s, _ = _scene(v, idx)
    dr = torch.from_numpy(rays).cuda()
    dh = torch.empty((n, 8), dtype=torch.int32, device="cuda")
    da = torch.empty(n, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    s.query_device(0, dr.data_ptr(), n, dh.data_ptr(), stream)
    s.query_device(1, dr.data_ptr(), n, da.data_ptr(), stream)
    torch.cuda.synchronize()
    want_h, want_a = dh.cpu().numpy().view(np.uint32), da.cpu().numpy().astype(bool)
    np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32).reshape(-1, 8), want_h)
    np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), want_a)
    # page-locked rays (read in place) and flags (written in place)
    from heavyrt_gb300 import engine as E

    pin = PinnedBuffer(rays.nbytes)
    pin_out = PinnedBuffer(n)
    pin.array(np.float32, rays.size)[:] = rays.reshape(-1)
    pinned_rays = pin.array(np.float32, rays.size).reshape(-1, 8)
    np.testing.assert_array_equal(s.RayQuery_NearestHit(pinned_rays).view(np.uint32).reshape(-1, 8), want_h)
    np.testing.assert_array_equal(s.RayQuery_AnyHit(pinned_rays), want_a)
    import ctypes

    s.ctx.check(E.lib().hrt_query_any_host(s._h, ctypes.c_void_p(pin.ptr), n, ctypes.c_void_p(pin_out.ptr)), "any")
    np.testing.assert_array_equal(pin_out.array(np.uint8, n).astype(bool), want_a)
    small = pinned_rays[:1000]
    np.testing.assert_array_equal(s.RayQuery_NearestHit(small).view(np.uint32).reshape(-1, 8), want_h[:1000])
    # asynchronous forms on two streams, page-locked and pageable arrays
    pin_hits = PinnedBuffer(32 * n)
    pageable_hits = np.zeros((n, 8), np.uint32)
    pageable_any = np.zeros(n, np.uint8)
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    L = E.lib()
    pin_out.array(np.uint8, n)[:] = 7
    assert L.hrt_query_nearest_host_async(s._h, ctypes.c_void_p(pin.ptr), n, ctypes.c_void_p(pin_hits.ptr),
                                          ctypes.c_void_p(sa.cuda_stream)) == 0
    assert L.hrt_query_any_host_async(s._h, ctypes.c_void_p(pin.ptr), n, ctypes.c_void_p(pin_out.ptr),
                                      ctypes.c_void_p(sb.cuda_stream)) == 0
    assert L.hrt_query_nearest_host_async(s._h, rays.ctypes.data_as(ctypes.c_void_p), n,
                                          pageable_hits.ctypes.data_as(ctypes.c_void_p),
                                          ctypes.c_void_p(sb.cuda_stream)) == 0
    assert L.hrt_query_any_host_async(s._h, rays.ctypes.data_as(ctypes.c_void_p), n,
                                      pageable_any.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(sa.cuda_stream)) == 0
    sa.synchronize()
    sb.synchronize()
    assert L.hrt_scene_check(s._h) == 0
    np.testing.assert_array_equal(pin_hits.array(np.uint32, 8 * n).reshape(-1, 8), want_h)
    np.testing.assert_array_equal(pin_out.array(np.uint8, n).astype(bool), want_a)
    np.testing.assert_array_equal(pageable_hits, want_h)
    np.testing.assert_array_equal(pageable_any.astype(bool), want_a)
    pin_hits.free()
    pin.free()
    pin_out.free()
    assert 0.2 < want_a.mean() < 1.0


def test_host_queries_in_place_and_alignment(native):
    """Page-locked rays and hits are read and written in place (nearest hits by
    the one-thread-per-ray kernel); records at a 32-byte boundary take one
    256-bit access, records at a 16-byte boundary two 128-bit ones; page-locked
    arrays off a 16-byte boundary go through the staging copies; every form
    gives the device query's results.  Arrays off a 16-byte boundary handed to
    the device entry points are refused before any launch (checked with n = 0,
    so that nothing could launch even if the check were missing)."""
    import ctypes

    import torch

    from heavyrt_gb300 import PinnedBuffer
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(8, 120, 120)
    rays = np.concatenate([wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 320, 200),
                           wl.rays_at_triangles(6, v, idx, 40001, jitter=0.02)])
    n = rays.shape[0]
    s, _ = _scene(v, idx)
    dr = torch.from_numpy(rays).cuda()
    dh = torch.empty((n, 8), dtype=torch.int32, device="cuda")
    da = torch.empty(n, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    s.query_device(0, dr.data_ptr(), n, dh.data_ptr(), stream)
    s.query_device(1, dr.data_ptr(), n, da.data_ptr(), stream)
    torch.cuda.synchronize()
    want_h, want_a = dh.cpu().numpy().view(np.uint32), da.cpu().numpy().astype(bool)
    L = E.lib()
    pin_r = PinnedBuffer(rays.nbytes + 64)
    pin_h = PinnedBuffer(32 * n + 64)
    pin_a = PinnedBuffer(n + 64)
    for r_off, h_off in ((0, 0), (16, 16), (0, 16), (16, 0), (4, 0), (0, 4)):
        pin_r.array(np.uint8, rays.nbytes + 64)[r_off:r_off + rays.nbytes] = rays.view(np.uint8).reshape(-1)
        hv = pin_h.array(np.uint8, 32 * n + 64)
        hv[:] = 0xAB
        rp, hp = ctypes.c_void_p(pin_r.ptr + r_off), ctypes.c_void_p(pin_h.ptr + h_off)
        assert L.hrt_query_nearest_host(s._h, rp, n, hp) == 0, (r_off, h_off, s.ctx.last_error())
        got = hv[h_off:h_off + 32 * n].view(np.uint32).reshape(-1, 8)
        np.testing.assert_array_equal(got, want_h, err_msg=f"rays +{r_off} B, hits +{h_off} B")
        assert (hv[:h_off] == 0xAB).all() and (hv[h_off + 32 * n:] == 0xAB).all()
        av = pin_a.array(np.uint8, n + 64)
        av[:] = 7
        assert L.hrt_query_any_host(s._h, rp, n, ctypes.c_void_p(pin_a.ptr + 1)) == 0
        np.testing.assert_array_equal(av[1:n + 1].astype(bool), want_a)
        assert av[0] == 7 and (av[n + 1:] == 7).all()
    # device entry points: off a 16-byte boundary is an invalid argument
    HRT_ERR_INVALID_ARGUMENT = 1
    assert L.hrt_query_nearest(s._h, ctypes.c_void_p(dr.data_ptr() + 4), 0, ctypes.c_void_p(dh.data_ptr()),
                               ctypes.c_void_p(stream)) == HRT_ERR_INVALID_ARGUMENT
    assert L.hrt_query_nearest(s._h, ctypes.c_void_p(dr.data_ptr()), 0, ctypes.c_void_p(dh.data_ptr() + 8),
                               ctypes.c_void_p(stream)) == HRT_ERR_INVALID_ARGUMENT
    assert L.hrt_query_any(s._h, ctypes.c_void_p(dr.data_ptr() + 8), 0, ctypes.c_void_p(da.data_ptr()),
                           ctypes.c_void_p(stream)) == HRT_ERR_INVALID_ARGUMENT
    assert "16-byte aligned" in s.ctx.last_error()
    # an any-hit output needs no alignment
    assert L.hrt_query_any(s._h, ctypes.c_void_p(dr.data_ptr()), 0, ctypes.c_void_p(da.data_ptr() + 1),
                           ctypes.c_void_p(stream)) == 0
    pin_r.free()
    pin_h.free()
    pin_a.free()


def test_instances_exact_transforms(native):
    """Several instances of one geometry; transforms exact in binary32 so the
    expected result is computed by tracing the oracle with transformed rays."""
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(12, 3000, off=0.05)
    mats = [np.eye(4, dtype=np.float32)]
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = [4.0, 0.0, 0.0]
    mats.append(m)
    m = np.diag([2.0, 2.0, 2.0, 1.0]).astype(np.float32)
    m[:3, 3] = [0.0, -8.0, 0.5]
    mats.append(m)
    rays = np.concatenate([wl.sphere_rays(4, 4000, 12.0),
                           wl.rays_at_triangles(5, v, idx, 2000, radius=6.0)])
    s, gid = _scene(v, idx, instances=mats)
    got = s.RayQuery_NearestHit(rays)
    o, _ = _oracle_expect(v, idx)
    best = np.empty(rays.shape[0], dtype=got.dtype)
    best["t"] = rays[:, 7]
    best["primId"] = best["instId"] = best["geomId"] = MISS
    best["coords"] = 0
    for k, mm in enumerate(mats):
        inv = np.linalg.inv(mm.astype(np.float64)).astype(np.float32)
        r = rays.copy()
        o3 = rays[:, 0:3].astype(np.float32)
        d3 = rays[:, 4:7].astype(np.float32)
        for row in range(3):
            a = inv[row]
            r[:, row] = ((a[0] * o3[:, 0] + a[1] * o3[:, 1]) + a[2] * o3[:, 2]) + a[3] * np.float32(1.0)
            r[:, 4 + row] = ((a[0] * d3[:, 0] + a[1] * d3[:, 1]) + a[2] * d3[:, 2]) + a[3] * np.float32(0.0)
        if k == 0:
            r = rays.copy()
        r[:, 7] = best["t"]
        h = o.trace(r)
        better = (h["geomId"] != MISS) & (h["t"] < best["t"])
        best[better] = h[better]
        best["instId"][better] = k
    found = best["geomId"] != MISS
    np.testing.assert_array_equal(got["geomId"] != MISS, found)
    np.testing.assert_array_equal(got["t"][found].view(np.uint32), best["t"][found].view(np.uint32))
    np.testing.assert_array_equal(got["instId"][found], best["instId"][found])
    np.testing.assert_array_equal(got["primId"][found], best["primId"][found])


@pytest.mark.parametrize("layout", ["bvh2", "bvh4_f16"])
def test_in_place_host_queries_with_instance_tree(native, layout):
    """Page-locked rays and results used in place on a scene of two instances
    (the two-level kernels: instance tree, one-thread-per-ray form for nearest
    hits) give the device query's results."""
    import ctypes

    import torch

    from heavyrt_gb300 import PinnedBuffer, SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(41, 8000, off=0.04)
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = [2.5, 0.0, 0.0]
    s = SceneRT(layout=layout)
    g = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
    s.AddInstance(g)
    s.AddInstance(g, m)
    s.CommitScene()
    rays = np.concatenate([wl.sphere_rays(3, 20000, 9.0), wl.rays_at_triangles(4, v, idx, 20000, radius=5.0)])
    n = rays.shape[0]
    dr = torch.from_numpy(rays).cuda()
    dh = torch.empty((n, 8), dtype=torch.int32, device="cuda")
    da = torch.empty(n, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    s.query_device(0, dr.data_ptr(), n, dh.data_ptr(), stream)
    s.query_device(1, dr.data_ptr(), n, da.data_ptr(), stream)
    torch.cuda.synchronize()
    want_h, want_a = dh.cpu().numpy().view(np.uint32), da.cpu().numpy().astype(bool)
    assert (want_h[:, 2] == 1).any() and (want_h[:, 2] == 0).any()  # hits on both instances
    pin_r, pin_h, pin_a = PinnedBuffer(rays.nbytes), PinnedBuffer(32 * n), PinnedBuffer(n)
    pin_r.array(np.float32, rays.size)[:] = rays.reshape(-1)
    L = E.lib()
    assert L.hrt_query_nearest_host(s._h, ctypes.c_void_p(pin_r.ptr), n, ctypes.c_void_p(pin_h.ptr)) == 0
    assert L.hrt_query_any_host(s._h, ctypes.c_void_p(pin_r.ptr), n, ctypes.c_void_p(pin_a.ptr)) == 0
    np.testing.assert_array_equal(pin_h.array(np.uint32, 8 * n).reshape(-1, 8), want_h)
    np.testing.assert_array_equal(pin_a.array(np.uint8, n).astype(bool), want_a)
    pin_r.free()
    pin_h.free()
    pin_a.free()
    s.close()


@pytest.mark.parametrize("layout", ["bvh2", "bvh4", "bvh4_f16", "bvh4_q8"])
def test_single_instance_transform_and_update(native, layout):
    """One instance: under a transform the scene takes the general kernel (the
    ray is mapped into the instance), after UpdateInstance to the identity and a
    new commit the single-instance kernel; both equal the oracle."""
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(31, 5000, off=0.04)
    m = np.diag([2.0, 2.0, 2.0, 1.0]).astype(np.float32)
    m[:3, 3] = [0.5, -1.0, 0.25]
    rays = np.concatenate([wl.sphere_rays(7, 3000, 8.0), wl.rays_at_triangles(8, v, idx, 3000, radius=4.0)])
    s = SceneRT(layout=layout)
    g = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
    s.AddInstance(g, m)
    s.CommitScene()
    o, _ = _oracle_expect(v, idx)
    inv = np.linalg.inv(m.astype(np.float64)).astype(np.float32)
    r = rays.copy()
    o3, d3 = rays[:, 0:3], rays[:, 4:7]
    for row in range(3):
        a = inv[row]
        r[:, row] = ((a[0] * o3[:, 0] + a[1] * o3[:, 1]) + a[2] * o3[:, 2]) + a[3] * np.float32(1.0)
        r[:, 4 + row] = ((a[0] * d3[:, 0] + a[1] * d3[:, 1]) + a[2] * d3[:, 2]) + a[3] * np.float32(0.0)
    want = o.trace(r)
    got = s.RayQuery_NearestHit(rays)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), o.trace(r, any_hit=True))
    assert (want["geomId"] != MISS).mean() > 0.2
    s.UpdateInstance(0, np.eye(4, dtype=np.float32))
    s.CommitScene()
    np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32), o.trace(rays).view(np.uint32))
    np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), o.trace(rays, any_hit=True))
    s.close()


def test_empty_geometry_and_errors(native):
    from heavyrt_gb300 import HrtError, SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    s = SceneRT()
    v = np.zeros((3, 4), np.float32)
    gid = s.AddGeom_Triangles3f(v, 3, np.zeros(0, np.uint32), 0, vByteStride=16)
    s.AddInstance(gid)
    with pytest.raises(HrtError) as e:
        s.RayQuery_NearestHit(wl.sphere_rays(1, 4))
    assert e.value.status == E.HRT_ERR_STATE  # query before commit
    s.CommitScene()
    h = s.RayQuery_NearestHit(wl.sphere_rays(1, 64))
    assert np.all(h["geomId"] == MISS) and np.all(h["t"] == np.float32(1e9))
    # index out of range
    with pytest.raises(HrtError) as e:
        s.AddGeom_Triangles3f(np.zeros((3, 4), np.float32), 3, np.array([0, 1, 5], np.uint32), 3, vByteStride=16)
    assert e.value.status == E.HRT_ERR_INVALID_ARGUMENT
    # more than 127 triangles with one Morton code: the reference's leaf count overflows
    tri = np.array([[0, 0, 0, 1], [1, 0, 0, 1], [0, 1, 0, 1]], dtype=np.float32)
    vv = np.concatenate([tri] * 300 + [tri + np.array([5, 5, 5, 0], np.float32)])
    with pytest.raises(HrtError) as e:
        s.AddGeom_Triangles3f(vv, vv.shape[0], np.arange(vv.shape[0], dtype=np.uint32), vv.shape[0], vByteStride=16)
    assert e.value.status == E.HRT_ERR_CAPACITY
    # a failed add leaves the scene usable
    assert s.GetGeomNum() == 1
    with pytest.raises(HrtError):
        SceneRT(build_name="cbvh_embree2")


def test_geom_boxes_and_info(native):
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(3, 1000)
    s, gid = _scene(v, idx)
    box = s.GetGeomBoxes()[gid]
    np.testing.assert_array_equal(box[:3], v[:, :3].min(axis=0))
    np.testing.assert_array_equal(box[4:7], v[:, :3].max(axis=0))
    info = s.geom_info(gid)
    assert info["tris"] == 1000 and info["leaves"] <= 1000 and info["build_ms"] > 0
    assert s.GetInstNum() == 1 and s.Name() == "GB300_LBVH"


def _walk_pairs(recs, peach):
    """Walks the engine's child-pair records and the reference's LEFT_OFFSET
    (peach) array side by side from the root: record r of the binary layout
    and the sibling pair at peach offset o hold the same two child boxes (bit
    for bit), the same leaf starts, and internal children map to each other.
    Returns the number of pairs compared."""
    LEAF = 0x80000000
    rec = recs.reshape(-1, 16)
    boxes = rec[:, :12].view(np.float32)
    refs = rec[:, 12:14]
    pb = np.stack([peach["boxMin"], peach["boxMax"]], axis=1).reshape(-1, 6)  # min xyz, max xyz
    seen = 0
    todo = [(0, 0)]
    while todo:
        r, o = todo.pop()
        seen += 1
        for c in (0, 1):
            eb = boxes[r, 6 * c:6 * c + 6]
            ref = int(refs[r, c])
            node_left = int(peach["leftOffset"][o + c])
            if ref == 0xFFFFFFFF:  # a lone leaf's empty slot: the reference's dummy node
                assert node_left == LEAF and int(peach["escapeIndex"][o + c]) == 0xFFFFFFFF
                continue
            np.testing.assert_array_equal(eb.view(np.uint32), pb[o + c].astype(np.float32).view(np.uint32))
            if ref & LEAF:
                assert node_left & LEAF
                assert (node_left & 0x00FFFFFF) == (ref & 0x00FFFFFF)  # leaf start (sorted position)
            else:
                assert not (node_left & LEAF)
                todo.append((ref, node_left))
    return seen


@pytest.mark.parametrize("n", [1, 2, 3, 257, 4097, 70001])
def test_pair_records_are_the_reference_sibling_pairs(native, n):
    """The binary layout's pair records hold the sibling pairs of the
    reference's LEFT_OFFSET array (core/builders/lbvh.cpp:492-729, the
    oracle's peach_convert): the same boxes and leaf starts, pair for pair,
    reached through the same child links."""
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(700 + n, n, off=0.05)
    o, _ = _oracle_expect(v, idx)
    s, gid = _scene(v, idx)
    recs = s.export(gid, E.EXPORT_PAIR_RECORDS)
    peach = o.peach_nodes()
    assert _walk_pairs(recs, peach) == max(o.n_leaves - 1, 1)
    s.close()
