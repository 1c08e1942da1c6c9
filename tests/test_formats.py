"""VSGF meshes through the C ABI (host-only calls, no GPU): round trips,
flag handling, malformed files, and HeavyRT's own meshes where present."""
import struct
from pathlib import Path

import numpy as np
import pytest


def _parse_vsgf(b: bytes):
    """Independent reader of the layout of examples/loader/cmesh.cpp:80-173."""
    size, nv, ni, nm, fl = struct.unpack_from("<QIIII", b, 0)
    o = 24
    pos = np.frombuffer(b, np.float32, 4 * nv, o).reshape(-1, 4)
    o += 16 * nv
    nrm = None
    if not fl & 8:
        nrm = np.frombuffer(b, np.float32, 4 * nv, o).reshape(-1, 4)
        o += 16 * nv
    if fl & 1:
        o += 16 * nv
    o += 8 * nv
    idx = np.frombuffer(b, np.uint32, ni, o)
    return size, pos, idx, nrm


def test_vsgf_round_trip(native, tmp_path):
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    v, idx, _ = wl.heightfield(3, 17, 11)
    E.save_vsgf(tmp_path / "h.vsgf", v, idx)
    b = (tmp_path / "h.vsgf").read_bytes()
    size, pos, pidx, nrm = _parse_vsgf(b)
    assert size == len(b) and nrm is None
    np.testing.assert_array_equal(pos, v)
    np.testing.assert_array_equal(pidx, idx)
    v2, i2, n2 = E.load_vsgf(tmp_path / "h.vsgf", normals=True)
    np.testing.assert_array_equal(v2, v)
    np.testing.assert_array_equal(i2, idx)
    assert not n2.any()


def test_vsgf_with_normals_and_tangents(native, tmp_path):
    from heavyrt_gb300 import engine as E

    rng = np.random.default_rng(0)
    nv, ni = 9, 12
    pos = rng.normal(size=(nv, 4)).astype(np.float32)
    nrm = rng.normal(size=(nv, 4)).astype(np.float32)
    tan = rng.normal(size=(nv, 4)).astype(np.float32)
    tex = rng.normal(size=(nv, 2)).astype(np.float32)
    idx = rng.integers(0, nv, ni).astype(np.uint32)
    body = pos.tobytes() + nrm.tobytes() + tan.tobytes() + tex.tobytes() + idx.tobytes() + np.zeros(4, np.uint32).tobytes()
    (tmp_path / "m.vsgf").write_bytes(struct.pack("<QIIII", 24 + len(body), nv, ni, 1, 1) + body)
    v, i, n = E.load_vsgf(tmp_path / "m.vsgf", normals=True)
    np.testing.assert_array_equal(v, pos)
    np.testing.assert_array_equal(n, nrm)
    np.testing.assert_array_equal(i, idx)


def test_vsgf_malformed(native, tmp_path):
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    with pytest.raises(E.HrtError):
        E.load_vsgf(tmp_path / "missing.vsgf")
    v, idx = wl.soup(1, 10)
    E.save_vsgf(tmp_path / "t.vsgf", v, idx)
    b = (tmp_path / "t.vsgf").read_bytes()
    (tmp_path / "cut.vsgf").write_bytes(b[:-20])
    with pytest.raises(E.HrtError):
        E.load_vsgf(tmp_path / "cut.vsgf")
    (tmp_path / "bad.vsgf").write_bytes(struct.pack("<QIIII", 24, 3, 4, 0, 8))  # 4 indices: not triangles
    with pytest.raises(E.HrtError):
        E.load_vsgf(tmp_path / "bad.vsgf")


def test_reference_meshes(native):
    """HeavyRT's own meshes (scenes/meshes/*.vsgf), where its sources are present."""
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import native_build

    ref = native_build.reference_root()
    if ref is None:
        pytest.skip("HeavyRT sources not present on this machine")
    meshes = sorted(Path(ref, "scenes", "meshes").glob("*.vsgf"))
    assert meshes
    for m in meshes:
        size, pos, idx, nrm = _parse_vsgf(m.read_bytes())
        v, i, n = E.load_vsgf(m, normals=True)
        np.testing.assert_array_equal(v, pos)
        np.testing.assert_array_equal(i, idx)
        if nrm is not None:
            np.testing.assert_array_equal(n, nrm)
        assert i.size % 3 == 0 and (i < len(v)).all()
