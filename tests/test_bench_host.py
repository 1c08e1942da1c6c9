"""Host-side logic of the benchmark that decides what its line reports: the
hit comparison that separates mismatches from ties, the mapping of sorted
triangle positions to original indices, the per-launch DRAM traffic read from
the committed ncu summaries, and the scalar copies of the sections' figures
in the line's config.  No GPU needed."""
import importlib.util
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
MISS = 0xFFFFFFFF


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rec(t, prim, inst=0, geom=0):
    r = np.zeros(8, np.uint32)
    r[0] = np.float32(t).view(np.uint32)
    r[1], r[2], r[3] = prim, inst, geom
    return r


def test_hit_diff_separates_mismatches_from_ties(bench):
    ref = np.stack([_rec(1.0, 5), _rec(2.0, 6), _rec(3.0, 7), _rec(4.0, 8), _rec(1e9, MISS, MISS, MISS),
                    _rec(5.0, 9)])
    hits = ref.copy()
    hits[1] = _rec(2.0 * (1 + 5e-6), 60)   # another triangle within 1e-5: a tie
    hits[2] = _rec(3.0, 70)                # another triangle at the same t: a tie, exact
    hits[3] = _rec(4.0 * (1 + 5e-5), 8)    # same triangle, t beyond 1e-5: a mismatch
    hits[4] = _rec(0.5, 1)                 # hit where the reference missed: a mismatch
    d = bench.hit_diff(hits, ref, "x")
    assert d == {"nearest_mismatch_vs_x": 2, "nearest_tie_vs_x": 2, "nearest_tie_exact_t_vs_x": 1}
    assert bench.hit_diff(ref, ref, "x")["nearest_mismatch_vs_x"] == 0


def test_to_original_maps_hits_only(bench):
    hits = np.stack([_rec(1.0, 0), _rec(1e9, MISS, MISS, MISS), _rec(2.0, 2)])
    out = bench.to_original(hits, np.array([7, 8, 9], np.uint32))
    assert out[:, 1].tolist() == [7, MISS, 9]
    assert hits[0, 1] == 0  # the input is not changed


def test_profile_traffic_reads_the_committed_summaries(bench):
    for name in ("trace_any_bvh4_f16_heightfield2M.txt", "trace_nearest_bvh4_f16_heightfield2M.txt"):
        v = bench.profile_traffic(name)
        assert v is not None and 1e8 < v < 1e9, name
    assert bench.profile_traffic("no_such_profile.txt") is None


def test_summarize_copies_section_figures(bench):
    line = {"config": {}, "plain": {"mrays_s": 3600.0},
            "batched": {"batched_mrays_s": 1900.0, "plain_mrays_s": 170.0, "speedup": 11.2,
                        "results_equal_plain": True},
            "precision": {"scenes": {"soup": {
                "t_error_vs_fp64": {"max_rel": 1e-4},
                "layouts": {"bvh2": {"mrays_s": 1500.0},
                            "bvh4_f16": {"mrays_s": 1670.0, "nearest_mismatch_vs_bvh2": 0,
                                         "anyhit_mismatch_vs_bvh2": 1}},
                "watertight": {"t_error_vs_fp64": {"max_rel": 5e-6},
                               "layouts": {"bvh2": {"mrays_s": 1400.0},
                                           "bvh4_f16": {"mrays_s": 1550.0, "nearest_mismatch_vs_bvh2": 2}}}}}}}
    bench.summarize(line)
    c = line["config"]
    assert c["plain_mrays_s"] == 3600.0
    assert c["batched_mrays_s"] == 1900.0 and c["batched_speedup"] == 11.2
    assert c["c2_soup_t_max_rel_vs_fp64"] == 1e-4 and c["c2_soup_bvh4_f16_mrays_s"] == 1670.0
    assert c["c2_soup_watertight_t_max_rel_vs_fp64"] == 5e-6
    assert c["c2_soup_watertight_bvh4_f16_mrays_s"] == 1550.0
    assert c["c2_hit_mismatches"] == 3  # every mismatch of either triangle test counts
