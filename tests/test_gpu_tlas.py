"""Instance tree (TLAS): queries over many instances give the results of the
instance-by-instance traversal (itself checked against the oracle), fetch
fewer nodes, and fall back to that traversal when the tree cannot be built."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _instances(n, seed, spread=20.0):
    rng = np.random.default_rng(seed)
    mats = []
    for _ in range(n):
        m = np.eye(4)
        m[:3, :3] = _rotation(rng) * rng.uniform(0.3, 1.5)
        m[:3, 3] = rng.uniform(-spread, spread, 3)
        mats.append(m.astype(np.float32))
    return mats


def _scene(geoms, inst, tlas, layout=0, merge=None):
    from heavyrt_gb300 import SceneRT

    s = SceneRT(layout=layout)
    if merge is not None:
        s.set_bvh4_merge(merge)
    s.set_tlas(tlas)
    gids = [s.AddGeom_Triangles3f(v, len(v), i, i.size, vByteStride=16) for v, i in geoms]
    for g, m in inst:
        s.AddInstance(gids[g], m)
    s.CommitScene()
    return s


def _geoms():
    from heavyrt_gb300 import workload as wl

    v1, i1 = wl.soup(31, 4000, off=0.05)
    v2, i2, _ = wl.heightfield(32, 40, 40)
    v3, i3 = wl.soup(33, 300, off=0.1)
    empty = (np.zeros((0, 4), np.float32), np.zeros(0, np.uint32))
    return [(v1, i1), (v2, i2), (v3, i3), empty]


def _rays(n, seed, spread=20.0):
    rng = np.random.default_rng(seed)
    o = rng.uniform(-spread - 5, spread + 5, (n, 3))
    t = rng.uniform(-spread, spread, (n, 3))
    d = t - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 4:7] = d
    r[:, 7] = 1e9
    r[::7, 3] = 0.5
    r[1::9, 7] = 8.0
    return r


def _compare(a, b):
    ha, hb = a.view(np.uint32).reshape(-1, 8), b.view(np.uint32).reshape(-1, 8)
    diff = np.any(ha != hb, axis=1)
    assert np.array_equal(ha[diff, 0], hb[diff, 0]), "a different hit distance"
    return int(diff.sum())  # exact ties between instances, resolved by visit order


@pytest.mark.parametrize("layout,merge", [(0, None), (2, 1), (3, 8)])
def test_tlas_matches_instance_loop(native, layout, merge):
    import torch

    geoms = _geoms()
    rng = np.random.default_rng(5)
    mats = _instances(600, 7)
    inst = [(int(rng.integers(len(geoms))), m) for m in mats]
    rays = _rays(30000, 9)
    on = _scene(geoms, inst, True, layout, merge)
    off = _scene(geoms, inst, False, layout, merge)
    h_on, h_off = on.RayQuery_NearestHit(rays), off.RayQuery_NearestHit(rays)
    assert (h_on["geomId"] != MISS).sum() > 3000  # the rays do hit
    assert _compare(h_on, h_off) == 0
    np.testing.assert_array_equal(on.RayQuery_AnyHit(rays), off.RayQuery_AnyHit(rays))
    # the instance tree visits far fewer nodes than testing every instance
    dr = torch.from_numpy(rays).cuda()
    p_on, _ = on.query_counters(0, dr.data_ptr(), len(rays))
    p_off, _ = off.query_counters(0, dr.data_ptr(), len(rays))
    assert p_on < p_off / 5


def test_tlas_vs_oracle_exact_transforms(native):
    """Translations and power-of-two scales (exact in binary32): the oracle
    traced with each instance's transformed rays, nearest over instances."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    v, idx = wl.soup(12, 3000, off=0.05)
    mats = []
    rng = np.random.default_rng(3)
    for k in range(40):
        m = np.eye(4, dtype=np.float32) * np.float32(2.0 ** int(rng.integers(-1, 2)))
        m[3, 3] = 1.0
        m[:3, 3] = rng.integers(-12, 13, 3).astype(np.float32)
        mats.append(m)
    s = _scene([(v, idx)], [(0, m) for m in mats], True)
    rays = _rays(20000, 4, 12.0)
    got = s.RayQuery_NearestHit(rays)
    o = orc.OracleBVH(v, idx)
    best = np.zeros((len(rays), 8), np.uint32)
    best[:, 0] = rays[:, 7].view(np.uint32)
    best[:, 1:4] = MISS
    bt = rays[:, 7].copy()
    for k, mm in enumerate(mats):
        inv = np.linalg.inv(mm.astype(np.float64)).astype(np.float32)
        r = rays.copy()
        o3, d3 = rays[:, 0:3], rays[:, 4:7]
        for row in range(3):
            a = inv[row]
            r[:, row] = ((a[0] * o3[:, 0] + a[1] * o3[:, 1]) + a[2] * o3[:, 2]) + a[3] * np.float32(1.0)
            r[:, 4 + row] = ((a[0] * d3[:, 0] + a[1] * d3[:, 1]) + a[2] * d3[:, 2]) + a[3] * np.float32(0.0)
        h = o.trace(r).view(np.uint32).reshape(-1, 8)
        ht = h[:, 0].view(np.float32)
        better = (h[:, 3] != MISS) & (ht < bt)
        best[better] = h[better]
        best[better, 2] = k
        bt[better] = ht[better]
    g = got.view(np.uint32).reshape(-1, 8)
    diff = np.any(g != best, axis=1)
    assert np.array_equal(g[diff, 0], best[diff, 0])  # only ties between instances may differ
    assert diff.sum() <= len(rays) // 1000
    assert (g[:, 3] != MISS).sum() > 1000


def test_tlas_coincident_instances(native):
    """200 identical instances share one Morton code: one instance-tree leaf
    longer than the 127 a geometry leaf may hold; the traversal walks it all
    and, with every t equal, the first instance wins as in instance order."""
    import torch

    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(2, 500, off=0.05)
    m = np.eye(4, dtype=np.float32)
    s = _scene([(v, idx)], [(0, m)] * 200, True)
    rays = wl.rays_at_triangles(1, v, idx, 2000, jitter=0.02)
    h = s.RayQuery_NearestHit(rays)
    one = _scene([(v, idx)], [(0, m)], True).RayQuery_NearestHit(rays)
    hit = h["geomId"] != MISS
    assert hit.sum() > 500
    assert np.all(h["instId"][hit] == 0)
    np.testing.assert_array_equal(h["t"].view(np.uint32), one["t"].view(np.uint32))
    np.testing.assert_array_equal(h["primId"], one["primId"])
    off = _scene([(v, idx)], [(0, m)] * 200, False)
    dr = torch.from_numpy(rays).cuda()
    # at most the tree's own (single-leaf) root record per ray on top of the 200 instance traversals
    p_on, _ = s.query_counters(0, dr.data_ptr(), len(rays))
    p_off, _ = off.query_counters(0, dr.data_ptr(), len(rays))
    assert p_off - len(rays) <= p_on <= p_off + len(rays)


def test_tlas_update_instance_and_recommit(native):
    geoms = _geoms()
    mats = _instances(50, 11, 8.0)
    inst = [(k % 3, m) for k, m in enumerate(mats)]
    s = _scene(geoms, inst, True)
    rays = _rays(5000, 12, 8.0)
    before = s.RayQuery_NearestHit(rays)
    moved = mats[7].copy()
    moved[:3, 3] += 3.0
    s.UpdateInstance(7, moved)
    s.CommitScene()
    inst2 = list(inst)
    inst2[7] = (inst[7][0], moved)
    ref = _scene(geoms, inst2, False)
    assert _compare(s.RayQuery_NearestHit(rays), ref.RayQuery_NearestHit(rays)) == 0
    assert not np.array_equal(before.view(np.uint32), s.RayQuery_NearestHit(rays).view(np.uint32))
