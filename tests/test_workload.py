"""Seeded scene / ray generators (CPU)."""
import numpy as np


def test_pcg32_known_answer(host_libs):
    # pcg32 with initstate 42, initseq 54: the first outputs of O'Neill's
    # reference implementation (pcg32-demo)
    from heavyrt_gb300 import workload as wl

    got = wl.pcg32(42, 54, 6)
    want = np.array([0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E], dtype=np.uint32)
    np.testing.assert_array_equal(got, want)


def test_soup_shape_and_range(host_libs):
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(1, 1000, -1.0, 1.0, 0.02)
    assert v.shape == (3000, 4) and idx.shape == (3000,)
    np.testing.assert_array_equal(idx, np.arange(3000))
    assert np.all(v[:, 3] == 1.0)
    c = v[:, :3].reshape(1000, 3, 3).mean(axis=1)
    assert np.all(np.abs(v[:, :3].reshape(1000, 3, 3) - c[:, None, :]) <= 0.04 + 1e-6)
    assert np.all(np.abs(v[:, :3]) <= 1.02 + 1e-6)
    v2, _ = wl.soup(1, 1000, -1.0, 1.0, 0.02)
    np.testing.assert_array_equal(v, v2)


def test_heightfield(host_libs):
    from heavyrt_gb300 import workload as wl

    v, idx, p = wl.heightfield(2, 16, 8)
    assert v.shape == (17 * 9, 4) and idx.shape == (6 * 16 * 8,)
    assert idx.max() == 17 * 9 - 1
    assert v[0, 0] == -1.0 and v[16, 0] == 1.0 and v[-1, 1] == 1.0
    assert np.all(np.abs(v[:, 2]) <= 0.2)  # sum of amplitudes 0.1 * (1 + 1/2 + ...) < 0.2


def test_camera_rays_normalised(host_libs):
    from heavyrt_gb300 import workload as wl

    r = wl.camera_rays((0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0, 32, 16, 0.0, 1e9)
    assert r.shape == (512, 8)
    n = np.linalg.norm(r[:, 4:7].astype(np.float64), axis=1)
    assert np.allclose(n, 1.0, atol=1e-6)
    assert np.all(r[:, 6] < 0)  # looking down -z
    assert np.all(r[:, 7] == np.float32(1e9))
    # vertical field of view: the top row's direction makes ~30 deg with -z
    top = r[16, 4:7]  # row 0, column 16
    assert abs(np.degrees(np.arctan2(top[1], -top[2])) - 30.0 * (15 / 16)) < 0.5


def test_ao_rays_leave_the_surface(host_libs):
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    v, idx, _ = wl.heightfield(4, 32, 32)
    eye = wl.camera_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, 64, 36)
    o = orc.OracleBVH(v, idx)
    hits = o.trace(eye)
    ao, owner = wl.ao_rays(3, eye, hits, v, o.sorted_indices(), 16, 0.2, 1e-4)
    nh = int((hits["geomId"] != 0xFFFFFFFF).sum())
    assert ao.shape == (16 * nh, 8)
    assert np.allclose(np.linalg.norm(ao[:, 4:7].astype(np.float64), axis=1), 1.0, atol=1e-6)
    assert np.all(ao[:, 7] == np.float32(0.2)) and np.all(ao[:, 3] == 0.0)
    # origins sit 1e-4 off the primary hit point
    e = eye[owner].astype(np.float64)
    hp = e[:, 0:3] + hits["t"][owner, None].astype(np.float64) * e[:, 4:7]
    off = np.linalg.norm(ao[:, 0:3] - hp, axis=1)
    assert np.all(off < 2e-4)
