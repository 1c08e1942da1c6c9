"""Speed of the oracle's restatement (the CPU baseline the benchmark times on
the GPU machine, kind "port") against the reference's own CPU traversal
compiled from its sources (oracle/_ref/ref_harness_fast: BVH2CommonRT's
BVH2TraverseC32, metrics off, OpenMP over rays), on the same machine, rays,
thread count and query: the benchmark frame's eye rays and AO rays, all traced
as nearest-hit queries (the reference answers any-hit through its nearest-hit
traversal, BVH2CommonRT::RayQuery_AnyHit being a stub).  Runs only where the
reference sources were compiled; prints one JSON line.

  python oracle/time_port_vs_reference.py [threads] [repeats]
"""
from __future__ import annotations

import json
import os
import platform
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def main():
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    threads = int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count()
    repeats = int(sys.argv[2]) if len(sys.argv) > 2 else 3
    exe = orc.reference_harness(fast=True)
    if exe is None:
        print(json.dumps({"unavailable": "reference checker not built here (reference sources absent)"}))
        return 0
    w = wl.config1()
    o = orc.OracleBVH(w.verts, w.idx)
    eye_hits = o.trace(w.eye_rays, threads=threads)
    ao = wl.frame_ao_rays(w, eye_hits, o.sorted_indices())
    rays = np.ascontiguousarray(np.concatenate([w.eye_rays, ao]))
    n = rays.shape[0]
    # the port: nearest-hit over every ray (best of `repeats`)
    port_s = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        hp = o.trace(rays, threads=threads)
        port_s.append(time.perf_counter() - t0)
    # the port's own any-hit traversal of the AO rays, as the benchmark times it
    t0 = time.perf_counter()
    o.trace(w.eye_rays, threads=threads)
    o.trace(ao, any_hit=True, threads=threads)
    port_bench_s = time.perf_counter() - t0
    # the reference: its harness times the traversal loop itself
    ref_ms = []
    with tempfile.TemporaryDirectory() as td:
        sp, rp, pre = os.path.join(td, "s.bin"), os.path.join(td, "r.bin"), os.path.join(td, "out")
        wl.scene_file(sp, w.verts, w.idx)
        wl.ray_file(rp, rays)
        for _ in range(repeats):
            r = subprocess.run([str(exe), "trace", sp, pre, rp, str(threads)], capture_output=True, text=True,
                               check=True)
            ref_ms.append(json.loads(r.stdout.strip().splitlines()[-1])["trace_ms"])
        hr = np.fromfile(pre + ".hits", dtype=orc.HIT_DTYPE)
    same = bool(np.array_equal(hr.view(np.uint32), hp.view(np.uint32)))
    ref_rate = n / (min(ref_ms) * 1e-3) / 1e6
    port_rate = n / min(port_s) / 1e6
    print(json.dumps({
        "workload": w.name, "rays": int(n), "eye_rays": int(len(w.eye_rays)), "ao_rays": int(len(ao)),
        "threads": threads, "cpu": platform.processor() or platform.machine(), "repeats": repeats,
        "query": "nearest hit for every ray (BVH2TraverseC32)",
        "reference_mrays_s": round(ref_rate, 3), "port_mrays_s": round(port_rate, 3),
        "port_over_reference": round(port_rate / ref_rate, 4),
        "port_benchmark_form_mrays_s": round(n / port_bench_s / 1e6, 3),
        "results_identical": same}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
