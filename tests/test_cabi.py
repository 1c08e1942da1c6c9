"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/hrt.h declares (no GPU work: this runs on the CPU-only machine too)."""
import ctypes
import re
from pathlib import Path

HEADER_DIR = Path(__file__).resolve().parents[1] / "include"


def declared_functions():
    names = set()
    for h in HEADER_DIR.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(hrt_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_the_interface():
    names = declared_functions()
    for must in ("hrt_scene_create", "hrt_add_geom_triangles3f", "hrt_commit_scene", "hrt_query_nearest",
                 "hrt_query_any", "hrt_add_instance", "hrt_clear_geom"):
        assert must in names


def test_library_exports_every_declared_symbol(native):
    lib = ctypes.CDLL(str(native["engine"]))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"libhrt.so lacks {missing}"


def test_host_only_entry_points(native):
    from heavyrt_gb300 import engine

    L = engine.lib()
    assert L.hrt_status_string(engine.HRT_ERR_CAPACITY).decode() == "format capacity exceeded"
    assert b"sm_103a" in L.hrt_version()
    # null arguments are rejected without touching a device
    assert L.hrt_context_create(0, None) == engine.HRT_ERR_INVALID_ARGUMENT
    assert L.hrt_scene_destroy(None) == engine.HRT_ERR_INVALID_ARGUMENT
    assert L.hrt_query_nearest(None, None, 0, None, None) == engine.HRT_ERR_INVALID_ARGUMENT


def test_engine_is_sm103a(native):
    from heavyrt_gb300 import native_build

    assert "arch=compute_103a,code=sm_103a" in native_build.ARCH


def test_rtao_sample_tile_is_host_code(native, host_libs):
    """hrt_rtao_qmc_table / hrt_rtao_qmc_tile run on the host: RTAO's quasi-random
    AO sample tile equals the oracle's (pinned against the reference's own
    generator by tests/test_oracle.py) for several sample counts."""
    import numpy as np
    from heavyrt_gb300 import engine
    from oracle import oracle as orc

    np.testing.assert_array_equal(engine.rtao_qmc_table(), orc.qmc_table())
    for r in (1, 2, 3, 4, 7, 16, 32):
        np.testing.assert_array_equal(engine.rtao_qmc_tile(r).view(np.uint32), orc.rtao_tile(r).view(np.uint32))
    L = engine.lib()
    assert L.hrt_rtao_qmc_tile(0, None) == engine.HRT_ERR_INVALID_ARGUMENT
    assert L.hrt_rtao_qmc_tile(engine.HRT_MAX_AO_RAYS_PER_PIXEL + 1, None) == engine.HRT_ERR_INVALID_ARGUMENT
    assert L.hrt_frame_destroy(None) == engine.HRT_ERR_INVALID_ARGUMENT
    assert L.hrt_frame_create(None, None) == engine.HRT_ERR_INVALID_ARGUMENT
