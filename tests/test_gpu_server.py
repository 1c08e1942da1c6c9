"""Serving loop: results are the same alone and in the mix, scenes uploaded
on arrival serve requests submitted before their build finished, and the
memory budget evicts idle scenes least recently used first."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF


def _scenes():
    from heavyrt_gb300 import workload as wl

    out = []
    for i, n in enumerate([1000, 7000, 30000, 300]):
        out.append(wl.soup(700 + i, n, off=0.03))
    for i, (nx, ny) in enumerate([(40, 30), (120, 100)]):
        v, idx, _ = wl.heightfield(710 + i, nx, ny)
        out.append((v, idx))
    return out


def _requests(scenes, count, seed):
    from heavyrt_gb300 import workload as wl

    rng = np.random.default_rng(seed)
    reqs = []
    for j in range(count):
        s = int(rng.integers(len(scenes)))
        kind = int(rng.integers(2))
        n = int(np.exp(rng.uniform(np.log(50), np.log(40000))))
        v, idx = scenes[s]
        r = np.concatenate([wl.rays_at_triangles(seed + j, v, idx, n - n // 4, jitter=0.03),
                            wl.sphere_rays(seed + j, n // 4)])
        reqs.append((s, kind, np.ascontiguousarray(r)))
    return reqs


def _out(kind, n):
    return np.empty((n, 8), np.uint32) if kind == 0 else np.empty(n, np.uint8)


def test_results_same_alone_and_in_the_mix(native):
    from heavyrt_gb300 import engine as E
    from oracle import oracle as orc

    scenes = _scenes()
    srv = E.Server(slot_rays=1 << 20, slots=3)
    ids = [srv.add_scene(v, idx, evictable=False) for v, idx in scenes]
    assert all(srv.scene_state(i, timeout=120) == E.SCENE_READY for i in ids)
    reqs = _requests(scenes, 60, 11)
    alone = []
    for s, kind, rays in reqs:
        out = _out(kind, len(rays))
        st, info = srv.wait(srv.submit_array(ids[s], kind, rays, out))
        assert st == 0 and info["batchRequests"] == 1
        alone.append(out)
    # the same requests submitted together from four threads
    outs = [_out(k, len(r)) for _, k, r in reqs]
    tickets = [None] * len(reqs)

    def submitter(t):
        for j in range(t, len(reqs), 4):
            s, kind, rays = reqs[j]
            tickets[j] = srv.submit_array(ids[s], kind, rays, outs[j])

    th = [threading.Thread(target=submitter, args=(t,)) for t in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    infos = []
    for j, t in enumerate(tickets):
        st, info = srv.wait(t)
        assert st == 0
        infos.append(info)
    for j in range(len(reqs)):
        np.testing.assert_array_equal(outs[j], alone[j], err_msg=f"request {j}")
    assert max(i["batchRequests"] for i in infos) > 1  # requests were batched together
    assert all(i["tSubmit"] <= i["tStart"] <= i["tDone"] for i in infos)
    # and they are the oracle's results
    for j in (0, 7, 23, 41):
        s, kind, rays = reqs[j]
        o = orc.OracleBVH(*scenes[s])
        if kind == 0:
            want = o.trace(rays).view(np.uint32).reshape(-1, 8).copy()
            hit = want[:, 1] != MISS
            want[hit, 2] = ids[s] & 0xFFFF
            want[hit, 3] = ids[s] & 0xFFFF
            np.testing.assert_array_equal(outs[j], want)
        else:
            np.testing.assert_array_equal(outs[j].astype(bool), o.trace(rays, any_hit=True))
    st = srv.stats()
    assert st["requests"] == 120 and st["failed"] == 0 and st["scenesResident"] == len(scenes)
    srv.close()


def test_page_locked_requests_are_traced_in_place(native):
    """Requests whose rays (and any-hit flags) sit in page-locked memory: a
    request batched alone is traced from them in place; results equal the
    same requests from pageable memory, alone and mixed into batches."""
    from heavyrt_gb300 import PinnedBuffer
    from heavyrt_gb300 import engine as E

    scenes = _scenes()
    srv = E.Server(slot_rays=1 << 20, slots=2)
    ids = [srv.add_scene(v, idx, evictable=False) for v, idx in scenes]
    assert all(srv.scene_state(i, timeout=120) == E.SCENE_READY for i in ids)
    reqs = _requests(scenes, 24, 29)
    want = []
    for s, kind, rays in reqs:
        out = _out(kind, len(rays))
        assert srv.wait(srv.submit_array(ids[s], kind, rays, out))[0] == 0
        want.append(out)
    bufs = []
    for s, kind, rays in reqs:
        pr, po = PinnedBuffer(rays.nbytes), PinnedBuffer(_out(kind, len(rays)).nbytes)
        pr.array(np.float32, rays.size)[:] = rays.reshape(-1)
        bufs.append((pr, po))
    # one at a time (each batched alone: read in place), then all at once (batched together)
    for rounds in range(2):
        tickets = []
        for j, (s, kind, rays) in enumerate(reqs):
            pr, po = bufs[j]
            po.array(np.uint8)[:] = 0xAB
            t = srv.submit(ids[s], kind, pr.ptr, len(rays), po.ptr)
            if rounds == 0:
                st, info = srv.wait(t)
                assert st == 0 and info["batchRequests"] == 1
            else:
                tickets.append(t)
        for t in tickets:
            assert srv.wait(t)[0] == 0
        for j, (s, kind, rays) in enumerate(reqs):
            got = bufs[j][1].array(np.uint32 if kind == 0 else np.uint8)
            np.testing.assert_array_equal(got.reshape(want[j].shape), want[j], err_msg=f"round {rounds} request {j}")
    for pr, po in bufs:
        pr.free()
        po.free()
    srv.close()


def test_upload_on_arrival(native):
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    srv = E.Server(slot_rays=1 << 18)
    v, idx = wl.soup(901, 150000, off=0.02)
    rays = wl.rays_at_triangles(4, v, idx, 50000, jitter=0.02)
    sid = srv.add_scene(v, idx)
    out = _out(1, len(rays))
    t = srv.submit_array(sid, 1, rays, out)  # queued while the scene builds
    st, info = srv.wait(t, 120.0)
    assert st == 0 and srv.scene_state(sid) == E.SCENE_READY
    np.testing.assert_array_equal(out.astype(bool), orc.OracleBVH(v, idx).trace(rays, any_hit=True))
    srv.close()


def test_budget_evicts_least_recently_used(native):
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(3, 20000, off=0.03)
    rays = wl.sphere_rays(2, 2000)
    # fixed costs and the size of one built scene, from a probe server
    probe = E.Server(slot_rays=1 << 16, slots=1)
    base = probe.stats()["residentBytes"]
    est = probe.scene_bytes(len(v), len(idx) // 3)
    probe.scene_state(probe.add_scene(v, idx), timeout=60)
    g = probe.stats()["residentBytes"] - base
    assert 0 < g <= est
    probe.close()
    srv = E.Server(slot_rays=1 << 16, slots=1, memory_budget=base + 3 * g + est - 1)
    a = srv.add_scene(v, idx, evictable=False)
    b = srv.add_scene(v, idx)
    c = srv.add_scene(v, idx)
    assert all(srv.scene_state(x, timeout=60) == E.SCENE_READY for x in (a, b, c))
    out = _out(0, len(rays))
    assert srv.wait(srv.submit_array(b, 0, rays, out))[0] == 0  # b is now more recent than c
    d = srv.add_scene(v, idx)  # does not fit: the least recently used idle evictable scene goes
    assert srv.scene_state(d, timeout=60) == E.SCENE_READY
    assert srv.scene_state(c) == E.SCENE_EVICTED
    assert srv.scene_state(a) == E.SCENE_READY and srv.scene_state(b) == E.SCENE_READY
    with pytest.raises(E.HrtError) as ei:
        srv.submit_array(c, 0, rays, out)
    assert ei.value.status == E.HRT_ERR_STATE
    st = srv.stats()
    assert st["evictions"] == 1 and st["residentBytes"] <= base + 3 * g + est - 1
    # a scene that cannot fit even after evicting everything evictable
    big_v, big_i = wl.soup(4, 400000, off=0.01)
    with pytest.raises(E.HrtError) as ei:
        srv.add_scene(big_v, big_i)
    assert ei.value.status == E.HRT_ERR_OUT_OF_MEMORY
    # removal
    srv.remove_scene(b)
    assert srv.scene_state(b) == E.SCENE_EVICTED
    srv.close()


def test_request_errors(native):
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(5, 500)
    srv = E.Server(slot_rays=4096, slots=2)
    sid = srv.add_scene(v, idx)
    rays = wl.sphere_rays(1, 5000)
    out = _out(0, len(rays))
    with pytest.raises(E.HrtError) as ei:
        srv.submit_array(sid, 0, rays, out)  # larger than a slot
    assert ei.value.status == E.HRT_ERR_CAPACITY
    with pytest.raises(E.HrtError):
        srv.submit(sid, 2, rays.ctypes.data, 10, out.ctypes.data)
    with pytest.raises(E.HrtError):
        srv.submit(sid ^ (1 << 16), 0, rays.ctypes.data, 10, out.ctypes.data)  # stale generation
    st, _ = srv.wait(12345)
    assert st == E.HRT_ERR_INVALID_ARGUMENT
    t = srv.submit(sid, 0, rays.ctypes.data, 0, out.ctypes.data)  # empty request
    assert srv.wait(t)[0] == 0
    srv.close()


def test_cubic_morton_frame_scenes(native):
    """A server configured with the cubic Morton frame builds every scene on
    that grid: binary-layout hits are the oracle's on the same grid bit for bit,
    any-hit flags are the reference's; a frame out of range is refused."""
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    with pytest.raises(E.HrtError):
        E.Server(slot_rays=4096, slots=1, morton_frame=7)
    srv = E.Server(slot_rays=1 << 18, slots=2, morton_frame=E.MORTON_CUBIC)
    scenes = _scenes()[:2] + _scenes()[4:]
    ids = [srv.add_scene(v, idx, evictable=False) for v, idx in scenes]
    assert all(srv.scene_state(i, timeout=120) == E.SCENE_READY for i in ids)
    for k, (v, idx) in enumerate(scenes):
        rays = np.concatenate([wl.rays_at_triangles(40 + k, v, idx, 3000, jitter=0.03), wl.sphere_rays(k, 1000)])
        oc = orc.OracleBVH(v, idx, cubic=True)
        want = oc.trace(rays).view(np.uint32).reshape(-1, 8).copy()
        hit = want[:, 1] != MISS
        want[hit, 2] = ids[k] & 0xFFFF
        want[hit, 3] = ids[k] & 0xFFFF
        out = _out(0, len(rays))
        assert srv.wait(srv.submit_array(ids[k], 0, rays, out))[0] == 0
        np.testing.assert_array_equal(out, want, err_msg=f"scene {k}")
        flags = _out(1, len(rays))
        assert srv.wait(srv.submit_array(ids[k], 1, rays, flags))[0] == 0
        np.testing.assert_array_equal(flags.astype(bool), orc.OracleBVH(v, idx).trace(rays, any_hit=True))
    srv.close()

    # 4-wide scenes on the cubic grid with the largest-first collapse: any-hit
    # flags are the reference's, nearest hits the oracle's on the same grid
    # up to ties within 1e-5 relative t
    srv = E.Server(slot_rays=1 << 18, slots=2, layout="bvh4_f16", bvh4_merge=1, morton_frame=E.MORTON_CUBIC,
                   bvh4_collapse=E.BVH4_COLLAPSE_LARGEST_FIRST)
    with pytest.raises(E.HrtError):
        E.Server(slot_rays=4096, slots=1, bvh4_collapse=5)
    ids = [srv.add_scene(v, idx, evictable=False) for v, idx in scenes]
    assert all(srv.scene_state(i, timeout=120) == E.SCENE_READY for i in ids)
    for k, (v, idx) in enumerate(scenes):
        rays = np.concatenate([wl.rays_at_triangles(60 + k, v, idx, 3000, jitter=0.03), wl.sphere_rays(k, 1000)])
        want = orc.OracleBVH(v, idx, cubic=True).trace(rays).view(np.uint32).reshape(-1, 8)
        out = _out(0, len(rays))
        assert srv.wait(srv.submit_array(ids[k], 0, rays, out))[0] == 0
        np.testing.assert_array_equal(out[:, 3] != MISS, want[:, 3] != MISS)
        same = out[:, 1] == want[:, 1]
        np.testing.assert_array_equal(out[same, 0], want[same, 0])
        tg, tw = out[~same, 0].view(np.float32).astype(np.float64), want[~same, 0].view(np.float32).astype(np.float64)
        assert np.all(np.abs(tg - tw) <= 1e-5 * np.abs(tw)) and np.count_nonzero(~same) <= 2
        flags = _out(1, len(rays))
        assert srv.wait(srv.submit_array(ids[k], 1, rays, flags))[0] == 0
        np.testing.assert_array_equal(flags.astype(bool), orc.OracleBVH(v, idx).trace(rays, any_hit=True))
    srv.close()
