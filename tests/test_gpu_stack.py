"""Short traversal stacks: the first S entries of a ray's stack in shared
memory, deeper entries spilled to local memory (hrt_trace_config.stackEntries).
Every S, far below and above the trees' depths, gives the same results as
the whole stack in shared memory, for every layout, both query kinds, both
launch forms, single-instance scenes and instance trees; and the oracle's."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

STACKS = [1, 2, 3, 4, 8, 16, 24, 32, 48, 64, 128]


def _scenes():
    from heavyrt_gb300 import workload as wl

    out = []
    g = dict(np.load(GOLDEN / "golden_duplicates40x5.npz"))
    out.append(("duplicates", g["verts"], g["idx"], g["rays"]))
    v, idx = wl.soup(51, 30000, off=0.05)
    out.append(("soup30000", v, idx, np.concatenate([wl.rays_at_triangles(6, v, idx, 4000, jitter=0.02),
                                                     wl.sphere_rays(7, 2000)])))
    hv, hidx, _ = wl.heightfield(9, 96, 96)
    rays = wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 96, 64)
    out.append(("heightfield96", hv, hidx, rays))
    return out


@pytest.mark.parametrize("layout", ["bvh2", "bvh4", "bvh4_f16", "bvh4_q8"])
def test_every_stack_size_gives_the_same_results(native, layout):
    from heavyrt_gb300 import SceneRT
    from oracle import oracle as orc

    for name, v, idx, rays in _scenes():
        o = orc.OracleBVH(v, idx)
        want_any = o.trace(rays, any_hit=True)
        s = SceneRT(layout=layout)
        if layout != "bvh2":
            s.set_bvh4_merge(1)
        gid = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
        s.AddInstance(gid)
        s.CommitScene()
        ref = s.RayQuery_NearestHit(rays).view(np.uint32)
        if layout == "bvh2":
            np.testing.assert_array_equal(ref.reshape(-1, 8), o.trace(rays).view(np.uint32).reshape(-1, 8))
        for stack in STACKS:
            for persistent in (1, 0):
                for kind in (0, 1):
                    s.set_trace_config(kind, 128, persistent, 16, 24, stack)
                np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32), ref,
                                              err_msg=f"{name} {layout} stack {stack}")
                np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), want_any, err_msg=f"{name} stack {stack}")
        s.close()


def test_short_stacks_with_instance_tree(native):
    """Two-level traversal (instance tree entries under each instance's own on
    one stack) with short stacks: the results of the whole stack."""
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(61, 4000, off=0.05)
    rng = np.random.default_rng(1)
    rays = wl.sphere_rays(2, 20000, 4.0)
    for layout in ("bvh2", "bvh4_f16"):
        s = SceneRT(layout=layout)
        gid = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
        for k in range(40):
            m = np.eye(4, dtype=np.float32)
            m[:3, :3] *= rng.uniform(0.2, 0.6)
            m[:3, 3] = rng.uniform(-2, 2, 3)
            s.AddInstance(gid, m)
        s.CommitScene()
        ref = s.RayQuery_NearestHit(rays).view(np.uint32)
        ref_any = s.RayQuery_AnyHit(rays)
        assert (ref_any != 0).sum() > 1000
        for stack in (1, 4, 16, 33, 64, 0):
            for persistent in (1, 0):
                for kind in (0, 1):
                    s.set_trace_config(kind, 64, persistent, 8, 16, stack)
                np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32), ref, err_msg=f"{stack}")
                np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), ref_any)
        s.close()


def test_stack_entries_out_of_range_refused(native):
    from heavyrt_gb300 import HrtError, SceneRT

    s = SceneRT()
    with pytest.raises(HrtError):
        s.set_trace_config(0, 128, 1, 16, 24, -1)
    with pytest.raises(HrtError):
        s.set_trace_config(0, 128, 1, 16, 24, 129)
    s.set_trace_config(0, 128, 1, 16, 24, 128)
    assert s.trace_config(0)["stackEntries"] == 128
    s.close()


@pytest.mark.parametrize("layout", ["bvh2", "bvh4_f16"])
def test_image_tile_order_gives_the_same_results(native, layout):
    """Rays taken in 4 x 8 pixel tiles of row-major images (imageWidth): the
    results of the given order, for widths that divide the ray count and that
    do not, in the single-instance, two-level and segmented kernels."""
    import torch

    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    hv, hidx, _ = wl.heightfield(9, 96, 96)
    rays = wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 203, 77)
    for n_inst in (1, 3):
        s = SceneRT(layout=layout)
        gid = s.AddGeom_Triangles3f(hv, hv.shape[0], hidx, hidx.size, vByteStride=16)
        for k in range(n_inst):
            m = np.eye(4, dtype=np.float32)
            m[2, 3] = 0.3 * k
            s.AddInstance(gid, m)
        s.CommitScene()
        ref = s.RayQuery_NearestHit(rays).view(np.uint32)
        ref_any = s.RayQuery_AnyHit(rays)
        assert ref_any.any()
        for width in (1, 7, 8, 203, 4096):
            for persistent in (1, 0):
                for kind in (0, 1):
                    s.set_trace_config(kind, 128, persistent, 16, 24, 0, width)
                np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32), ref,
                                              err_msg=f"{n_inst} {width} {persistent}")
                np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), ref_any)
        # segmented launch over the scene's instances with the tile order
        if n_inst == 3:
            dr = torch.from_numpy(rays).cuda()
            offs = np.array([0, 5000, 9000, len(rays)], np.uint32)
            do = torch.from_numpy(offs.view(np.int32)).cuda()
            ds = torch.from_numpy(np.array([2, 0, 1], np.int32)).cuda()
            outs = []
            for width in (0, 203):
                s.set_trace_config(0, 128, 1, 16, 24, 0, width)
                out = torch.zeros((len(rays), 8), dtype=torch.int32, device="cuda")
                s.query_multi(E.query_desc(0, dr.data_ptr(), len(rays), out.data_ptr(), do.data_ptr(),
                                           ds.data_ptr(), 3))
                torch.cuda.synchronize()
                outs.append(out.cpu().numpy())
            np.testing.assert_array_equal(outs[0], outs[1])
        s.close()


def test_l2_persisting_window_keeps_results(native):
    """A persisting-L2 window over a single-instance scene's nodes
    (HRT_OPTION_L2_PERSIST) changes no result; out-of-range sizes are refused;
    turning it off restores the context's set-aside."""
    from heavyrt_gb300 import HrtError, SceneRT
    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(13, 128, 128)
    rays = np.concatenate([wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 160, 90),
                           wl.rays_at_triangles(4, v, idx, 4000, jitter=0.02)])
    for layout in ("bvh2", "bvh4_f16"):
        s = SceneRT(layout=layout)
        gid = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
        s.AddInstance(gid)
        s.CommitScene()
        ref = s.RayQuery_NearestHit(rays).view(np.uint32)
        ref_any = s.RayQuery_AnyHit(rays)
        for mib in (1, 64, 0):
            s.set_l2_persist(mib)
            np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32), ref)
            np.testing.assert_array_equal(s.RayQuery_AnyHit(rays), ref_any)
        with pytest.raises(HrtError):
            s.set_l2_persist(-1)
        s.close()
