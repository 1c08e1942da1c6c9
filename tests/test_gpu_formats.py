"""BVH blobs restore a geometry without a build (identical arrays and
results), only into a scene of the same layout; a VSGF mesh traces like the
oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("layout,merge", [(0, None), (2, 1), (3, 8)])
def test_blob_round_trip(native, tmp_path, layout, merge):
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(9, 70, 60)
    a = SceneRT(layout=layout)
    if merge is not None:
        a.set_bvh4_merge(merge)
    g = a.AddGeom_Triangles3f(v, len(v), idx, idx.size, vByteStride=16)
    a.AddInstance(g)
    a.CommitScene()
    a.save_geom(g, tmp_path / "g.bvh")
    b = SceneRT(layout=layout)
    gb = b.load_geom(tmp_path / "g.bvh")
    b.AddInstance(gb)
    b.CommitScene()
    whats = list(range(9)) + ([E.EXPORT_NODES4] if layout else [])
    for what in whats:
        np.testing.assert_array_equal(a.export(g, what).view(np.uint8), b.export(gb, what).view(np.uint8))
    rays = np.concatenate([wl.rays_at_triangles(1, v, idx, 4000, jitter=0.02), wl.sphere_rays(2, 1000)])
    np.testing.assert_array_equal(a.RayQuery_NearestHit(rays).view(np.uint32), b.RayQuery_NearestHit(rays).view(np.uint32))
    np.testing.assert_array_equal(a.RayQuery_AnyHit(rays), b.RayQuery_AnyHit(rays))
    np.testing.assert_array_equal(a.GetGeomBoxes(), b.GetGeomBoxes())
    other = SceneRT(layout=(layout + 1) % 4)
    with pytest.raises(E.HrtError) as ei:
        other.load_geom(tmp_path / "g.bvh")
    assert ei.value.status == E.HRT_ERR_STATE
    blob = (tmp_path / "g.bvh").read_bytes()
    (tmp_path / "cut.bvh").write_bytes(blob[: len(blob) // 2])
    with pytest.raises(E.HrtError):
        SceneRT(layout=layout).load_geom(tmp_path / "cut.bvh")
    # a blob of another format version is refused by name
    assert blob[:6] == b"HRTBVH"
    (tmp_path / "old.bvh").write_bytes(blob[:6] + b"01" + blob[8:])
    c = SceneRT(layout=layout)
    with pytest.raises(E.HrtError):
        c.load_geom(tmp_path / "old.bvh")
    assert "format version" in c.ctx.last_error()


def test_vsgf_mesh_traces_like_oracle(native, tmp_path):
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    v, idx, _ = wl.heightfield(12, 40, 40)
    E.save_vsgf(tmp_path / "m.vsgf", v, idx)
    mv, mi = E.load_vsgf(tmp_path / "m.vsgf")
    s = SceneRT()
    g = s.AddGeom_Triangles3f(mv, len(mv), mi, mi.size, vByteStride=16)
    s.AddInstance(g)
    s.CommitScene()
    rays = wl.rays_at_triangles(3, v, idx, 3000, jitter=0.02)
    np.testing.assert_array_equal(s.RayQuery_NearestHit(rays).view(np.uint32),
                                  orc.OracleBVH(mv, mi).trace(rays).view(np.uint32))
