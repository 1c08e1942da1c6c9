"""Benchmark: Mrays/s of nearest-hit + any-hit queries on one GB300.

Workload (one "step" = one frame of HeavyRT's RTAO renderer on the
1024 x 1024-quad heightfield, 2,097,152 triangles):
  * 1920 x 1080 eye rays, RayQuery_NearestHit;
  * 16 cosine-weighted AO rays per primary hit, RayQuery_AnyHit.
value = (eye rays + AO rays) / step time, inputs resident in HBM, on the
        quantised-node scene (BVH4 FP16) with autotuned launch shapes;
        "plain" = the binary FP32 tree (the reference's decisions) on the same rays.
e2e   = the same through the host-pointer C-ABI calls: every step copies the
        step's rays from pinned host memory and the results back;
        e2e_device_raygen = the frame with its rays made on the device.
Further sections of the same JSON line: "frames" (whole frames of the example
renderers, RTAO and eye rays, generated, traced and shaded on the device),
"batched" (256 scenes, segmented build
and graph-captured launches vs per-scene plain), "served" (request stream over
64 resident scenes: p50/p99 vs one-at-a-time plain), "precision" (heightfield
+ 8.4M-triangle soup in every node layout, hit agreement, FP64 t error).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference's CPU algorithm (the oracle restatement
of HeavyRT's BVH2CommonRT traversal, OpenMP over rays on every host core) on
the same frame.  N > 1 (torchrun) runs independent replicas, one per GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s nearest/any-hit on 1 GB300, served+batched vs plain; p99 latency"
UNIT = "Mrays/s"
FALLBACK_HBM_GBS = 6800.0
LAYOUT_NODE_BYTES = {"bvh2": 64, "bvh4": 128, "bvh4_f16": 64, "bvh4_q8": 64}  # bytes per node fetch
LAYOUT_DESC = {"bvh2": "BVH2 pair records (64 B) + sorted triangle records",
               "bvh4": "BVH4 FP32 nodes (128 B) + sorted triangle records",
               "bvh4_f16": "BVH4 FP16 nodes rounded outward (64 B) + sorted triangle records",
               "bvh4_q8": "BVH4 8-bit nodes in per-node frames (64 B) + sorted triangle records"}
TRI_BYTES = 36         # three float3 (vertex A and two edges)
RAY_BYTES = 32         # {posAndNear, dirAndFar}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=300)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="engine", choices=["engine", "reference"])
    p.add_argument("--nx", type=int, default=1024, help="heightfield quads per side")
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU-baseline sample length")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--layout", default="bvh4_f16", choices=["bvh2", "bvh4", "bvh4_f16", "bvh4_q8"],
                   help="node layout of the headline scene (binary FP32, 4-wide FP32/FP16/8-bit)")
    p.add_argument("--merge", type=int, default=1, help="BVH4 leaf merge bound of the headline scene")
    p.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    p.add_argument("--launch-nearest", default=None,
                   help="launch shape of the nearest-hit kernel, 'threads,persistent,steps,lanes' (skips its tuning)")
    p.add_argument("--launch-any", default=None, help="launch shape of the any-hit kernel (as --launch-nearest)")
    p.add_argument("--no-plain", action="store_true", help="skip the plain BVH2 FP32 comparison")
    p.add_argument("--ncu", action="store_true",
                   help="profiling run: setup, warm-up and timed steps only (no extra builds, counters, e2e, CPU)")
    p.add_argument("--no-frames", action="store_true", help="skip the example renderers' device frames")
    p.add_argument("--only-frames", action="store_true", help="only the example renderers' device frames")
    p.add_argument("--no-batched", action="store_true", help="skip the 256-scene batched measurement")
    p.add_argument("--only-batched", action="store_true",
                   help="run only the 256-scene batched measurement (prints its JSON object)")
    p.add_argument("--batch-scenes", type=int, default=256)
    p.add_argument("--no-precision", action="store_true", help="skip the quantised-node precision measurement")
    p.add_argument("--only-precision", action="store_true",
                   help="run only the quantised-node precision measurement (prints its JSON object)")
    p.add_argument("--soup-tris", type=int, default=8388608, help="soup size of the precision measurement")
    p.add_argument("--only-build", type=int, default=0, metavar="K",
                   help="only K builds of the headline scene (the launch list of the build)")
    p.add_argument("--only-build-batched", type=int, default=0, metavar="K",
                   help="only K segmented builds of the 256-soup batch, BVH4 FP16 merge 1 (its launch list)")
    p.add_argument("--no-watertight", action="store_true", help="skip the watertight triangle-test measurement")
    p.add_argument("--morton-frame", default="cubic", choices=["cubic", "per_axis"],
                   help="Morton grid of the headline scene: cubic cells (engine option) or the reference's per-axis grid")
    p.add_argument("--bvh4-collapse", default="largest_first", choices=["largest_first", "even_depth"],
                   help="4-wide collapse of the headline scene: largest subtrees opened first (engine option) or "
                        "the reference's even-depth rule")
    p.add_argument("--split", default="replicas", choices=["replicas", "rays"],
                   help="N > 1: every rank traces the whole frame (replicas, weak scaling) or its share of the "
                        "frame's eye and AO rays, results gathered on rank 0 through host memory (strong scaling)")
    p.add_argument("--no-frame-compare", action="store_true",
                   help="skip timing the headline layout on the reference's own tree (per-axis grid, even-depth "
                        "collapse) and with the even-depth collapse alone")
    p.add_argument("--eye-order", default="tiles", choices=["tiles", "given"],
                   help="eye rays traced in 4x8 pixel tiles of the image (index arithmetic) or in the order given")
    p.add_argument("--l2-persist", type=int, default=64, metavar="MIB",
                   help="persisting-L2 window over the headline scene's nodes (MiB set aside; 0 none) for the "
                        "timed region and the end-to-end leg")
    p.add_argument("--no-l2-sweep", action="store_true", help="skip the persisting-L2 window sweep")
    p.add_argument("--no-oracle-check", action="store_true",
                   help="skip the check of every ray of the headline frame against the oracle")
    p.add_argument("--no-served", action="store_true", help="skip the served-stream measurement")
    p.add_argument("--only-served", action="store_true",
                   help="run only the served-stream measurement (prints its JSON object)")
    p.add_argument("--served-seconds", type=float, default=4.0, help="length of the request arrival trace")
    p.add_argument("--served-rate", type=float, default=2000.0, help="Poisson arrival rate, requests/s")
    return p.parse_args()


def dist_env():
    from heavyrt_gb300 import replicas

    r = replicas.from_env()
    return r.rank, r.world, r.local


def measured_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(name: str):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch_full:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap,temperature.gpu")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}

    def spread(self) -> dict:
        """SM clock spread and GPU temperature over the samples taken (call after stop)."""
        sm, temp = [], []
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                sm.append(float(parts[1]))
                temp.append(float(parts[9]))
            except ValueError:
                continue
        if not sm:
            return {}
        return {"sm_mhz_p10": float(np.percentile(sm, 10)), "sm_mhz_median": float(np.median(sm)),
                "temp_c_median": float(np.median(temp)), "samples": len(sm)}


def build_bytes(n_tris: int, n_verts: int, n_leaves: int, n_nodes4: int, node4_bytes: int) -> int:
    """Algorithmic bytes of one LBVH build (reads + writes of each stage, as the
    build kernels touch them): scene box 16 B per vertex; Morton codes 12 B
    indices + 48 B vertex gathers + 8 B pair out per triangle, plus the 8 B
    copy of the unsorted codes; radix sort 4 digit passes x (8 B in + 8 B out)
    + 4 B histogram read per pair; run compaction 4 B per code in + 8 B per run
    out; leaves 4 + 12 + 48 + 48 + 12 B per triangle + 32 B per leaf; Karras
    hierarchy 2 log2(L) code reads + 16 B out per internal node; refit 2 x 32 B
    + 2 x 4 B in, 32 B + 4 B out per internal node; then for the binary layout
    pair records 96 B in + 64 B out per internal node, for a 4-wide layout the
    collapse: 9 B of plan arrays per internal node + 4 x 32 B in + one node out
    per 4-wide node."""
    import math

    internal = max(n_leaves - 1, 0)
    log_l = math.log2(max(n_leaves, 2))
    return int(16 * n_verts + n_tris * (12 + 48 + 8 + 8) + n_tris * (4 * 16 + 4) + 4 * n_tris + 8 * n_leaves
               + n_tris * (4 + 12 + 48 + 48 + 12) + 32 * n_leaves + internal * (8 * log_l + 16)
               + internal * (64 + 8 + 32 + 4)
               + (internal * 9 + n_nodes4 * (4 * 32 + node4_bytes) if n_nodes4 else internal * (96 + 64)))


def make_frame(args):
    """Scene + eye rays of the heightfield RTAO frame (host arrays)."""
    from heavyrt_gb300 import workload as wl

    w = wl.config1(args.nx, args.width, args.height)
    return w


def ao_from_hits(w, hits, sorted_idx):
    from heavyrt_gb300 import workload as wl

    p = w.params
    ao, _ = wl.ao_rays(p["ao_seed"], w.eye_rays, hits, w.verts, sorted_idx, p["ao_per_hit"], p["ao_length"],
                       p["ao_offset"])
    return ao


# ---------------------------------------------------------------- CPU (reference algorithm)

def cpu_trace_rate(o, eye, ao, seconds: float, threads: int = 0):
    """Mrays/s of the oracle traversal over a bounded sample of the frame
    (eye and AO rays in the frame's proportion)."""
    n_eye, n_ao = eye.shape[0], ao.shape[0]
    frac = 0.02
    t0 = time.perf_counter()
    e_s = eye[: max(1, int(n_eye * frac))]
    a_s = ao[:: max(1, int(1 / frac))]
    o.trace(e_s, threads=threads)
    o.trace(a_s, any_hit=True, threads=threads)
    dt = time.perf_counter() - t0
    rate = (e_s.shape[0] + a_s.shape[0]) / dt
    # sample size for the target duration: part of the frame, or whole frames repeated
    frac = min(1.0, seconds * rate / (n_eye + n_ao))
    reps = max(1, int(seconds * rate / (n_eye + n_ao))) if frac >= 1.0 else 1
    e_s = eye[: max(1, int(n_eye * frac))]
    step = max(1, int(round(1 / frac))) if frac < 1.0 else 1
    a_s = ao[::step]
    t0 = time.perf_counter()
    for _ in range(reps):
        _, _, used = o.trace(e_s, threads=threads, counters=True)
        o.trace(a_s, any_hit=True, threads=threads)
    dt = time.perf_counter() - t0
    n = (e_s.shape[0] + a_s.shape[0]) * reps
    return n / dt / 1e6, used, f"{reps} x ({e_s.shape[0]} eye rays (first rows) + {a_s.shape[0]} AO rays " \
                               f"(every {step}th)) of the frame, {dt:.1f} s"


def host_cpu() -> str:
    """The host CPU's model name and logical core count (for the CPU-baseline record)."""
    name = ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware") and ":" in line:
                    name = line.split(":", 1)[1].strip()
                    break
                if key == "cpu part" and not name and ":" in line:
                    name = "Arm CPU part " + line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return f"{name or platform.processor() or platform.machine()} ({os.cpu_count()} logical cores)"


# Speed of the restatement against the reference's own traversal compiled from
# its sources (oracle/time_port_vs_reference.py: the frame's 6,073,008 rays,
# nearest hit for every ray, identical results, same machine and threads).
# The reference's sources exist only where the checker is built, so the factor
# is a recorded measurement: the port runs this much faster than the
# reference, i.e. the reference itself would be this much slower than the
# CPU baseline reported here.
PORT_OVER_REFERENCE = {"min": 1.08, "max": 1.21, "machine": "x86-64 Xeon @ 2.7 GHz, 8 and 1 threads",
                       "script": "oracle/time_port_vs_reference.py"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as orc

    w = make_frame(args)
    o = orc.OracleBVH(w.verts, w.idx)
    eye_hits = o.trace(w.eye_rays)
    ao = ao_from_hits(w, eye_hits, o.sorted_indices())
    n_eye, n_ao = w.eye_rays.shape[0], ao.shape[0]
    # each step: a bounded sample of the frame, eye and AO rays in proportion
    per_step = max(1.0, min(20.0, 120.0 / max(1, args.steps + args.warmup)))
    rate0, used, _ = cpu_trace_rate(o, w.eye_rays, ao, 1.0)
    frac = min(1.0, per_step * rate0 * 1e6 / (n_eye + n_ao))
    e_s = w.eye_rays[: max(1, int(n_eye * frac))]
    stride = max(1, int(round(1 / frac))) if frac < 1.0 else 1
    a_s = ao[::stride]
    for _ in range(args.warmup):
        o.trace(e_s)
        o.trace(a_s, any_hit=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.trace(e_s)
        o.trace(a_s, any_hit=True)
    dt = time.perf_counter() - t0
    n = (e_s.shape[0] + a_s.shape[0]) * args.steps
    value = n / dt / 1e6
    sample = (f"per step {e_s.shape[0]} of {n_eye} eye rays + {a_s.shape[0]} of {n_ao} AO rays "
              f"(every {stride}th); oracle restatement of BVH2CommonRT, OpenMP over rays")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w.name, "tris": int(w.idx.size // 3), "eye_rays": int(n_eye), "ao_rays": int(n_ao),
                   "parallelism": "cpu", "l2": "n/a (host)"},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": int(used), "kind": "port", "sample": sample,
                         "cpu": host_cpu(), "port_over_reference": PORT_OVER_REFERENCE},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- batched scenes

def run_batched(ctx, args, tune: bool = True) -> dict:
    """256 independent soups (log-uniform 1k..256k triangles) with log-uniform
    4k..64k rays each: one segmented build + one graph-captured launch per
    query kind over all scenes ("batched"), against one build and two
    launches per scene ("plain": BVH2 FP32, default launch shape)."""
    import torch

    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import autotune as AT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    w = wl.config3(args.batch_scenes)
    G = len(w.verts)
    n = int(w.ray_offsets[-1])
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    d_rays = torch.from_numpy(w.rays).cuda()
    d_offs = torch.from_numpy(w.ray_offsets.view(np.int32)).cuda()
    seg_inst = AT.seg_inst_identity(G)
    d_seg = torch.from_numpy(seg_inst.view(np.int32)).cuda()
    d_hits = torch.empty((n, 8), dtype=torch.int32, device="cuda")
    d_any = torch.empty(n, dtype=torch.uint8, device="cuda")

    # structure + launch shape
    if tune and not args.ncu:
        tr = AT.tune_batch(ctx, w.verts, w.idx, d_rays.data_ptr(), n, d_offs.data_ptr(), d_seg.data_ptr(), G,
                           d_hits.data_ptr(), d_any.data_ptr())
        layout, merge, collapse = tr.layout, tr.merge, tr.collapse
    else:
        tr, layout, merge, collapse = None, "bvh4_f16", 1, AT.EVEN

    # batched build: repeated for timing (GPU time of the whole batch)
    b_ms, b_wall = [], []
    for _ in range(1 if args.ncu else 3):
        t0 = time.perf_counter()
        scene, ids = AT.build_batch(ctx, w.verts, w.idx, layout, merge, collapse)
        b_wall.append(time.perf_counter() - t0)
        b_ms.append(scene.geom_info(ids[0])["build_ms"])
        if _ < (0 if args.ncu else 2):
            scene.close()
    if tr is not None:
        AT.apply(scene, tr)
    descs = [E.query_desc(0, d_rays.data_ptr(), n, d_hits.data_ptr(), d_offs.data_ptr(), d_seg.data_ptr(), G),
             E.query_desc(1, d_rays.data_ptr(), n, d_any.data_ptr(), d_offs.data_ptr(), d_seg.data_ptr(), G)]
    graph = scene.capture(descs)
    steps = max(3, args.steps // 10)
    for _ in range(3):
        graph.launch(sh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        graph.launch(sh)
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1) / steps
    if args.ncu:
        graph.close()
        return {"ncu_run": True, "batched_ms": batched_ms}
    hits_b = d_hits.cpu().numpy().view(np.uint32)
    any_b = d_any.cpu().numpy()

    # plain: one scene per soup, one build and two launches per scene
    plain, p_ms = [], []
    t0 = time.perf_counter()
    for i in range(G):
        s = SceneRT(ctx)
        g = s.AddGeom_Triangles3f(w.verts[i], len(w.verts[i]), w.idx[i], w.idx[i].size, vByteStride=16)
        s.AddInstance(g)
        s.CommitScene()
        p_ms.append(s.geom_info(g)["build_ms"])
        plain.append(s)
    p_wall = time.perf_counter() - t0
    p_hits = torch.empty_like(d_hits)
    p_any = torch.empty_like(d_any)
    offs = w.ray_offsets.astype(np.int64)

    def plain_step(evs=None):
        for i, s in enumerate(plain):
            a, b = int(offs[i]), int(offs[i + 1])
            if evs is not None:
                evs[i][0].record(stream)
            s.query_device(0, d_rays.data_ptr() + 32 * a, b - a, p_hits.data_ptr() + 32 * a, sh)
            s.query_device(1, d_rays.data_ptr() + 32 * a, b - a, p_any.data_ptr() + a, sh)
            if evs is not None:
                evs[i][1].record(stream)

    for _ in range(2):
        plain_step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        plain_step()
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / steps
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(G)]
    plain_step(evs)
    torch.cuda.synchronize()
    plain_kernel_ms = sum(a.elapsed_time(b) for a, b in evs)
    # the batched results are the per-scene results, up to the instance id (scene index)
    ph = p_hits.cpu().numpy().view(np.uint32).copy()
    hit = ph[:, 1] != 0xFFFFFFFF
    owner = np.repeat(np.arange(G, dtype=np.uint32), np.diff(offs))
    ph[hit, 2] = owner[hit]
    ph[hit, 3] = owner[hit]
    same = bool(np.array_equal(ph, hits_b) and np.array_equal(p_any.cpu().numpy(), any_b))
    graph.close()
    scene.close()
    for s in plain:
        s.close()
    rays2 = 2 * n  # each ray is traced twice: nearest and any
    out = {
        "workload": w.name, "scenes": G, "tris": w.params["tris"], "rays": n,
        "structure": {"layout": layout, "bvh4_merge": merge,
                      "bvh4_collapse": ("largest_first" if collapse == AT.LARGEST else "even_depth")
                      if layout != "bvh2" else None},
        "launch": tr.configs if tr is not None else None,
        "tuning_table_ms": tr.table if tr is not None else None,
        "batched_mrays_s": round(rays2 / batched_ms / 1e3, 2), "batched_ms": round(batched_ms, 4),
        "plain_mrays_s": round(rays2 / plain_ms / 1e3, 2), "plain_ms": round(plain_ms, 4),
        "plain_kernel_sum_ms": round(plain_kernel_ms, 4),
        "speedup": round(plain_ms / batched_ms, 2),
        "build_batched_gpu_ms": round(statistics.median(b_ms), 3),
        "build_batched_wall_ms": round(1e3 * statistics.median(b_wall), 1),
        "build_plain_gpu_ms_sum": round(sum(p_ms), 3), "build_plain_wall_ms": round(1e3 * p_wall, 1),
        "results_equal_plain": same,
        "note": "batched = segmented build + one CUDA graph of two segmented launches (nearest, any) over all "
                "scenes, structure and launch shape autotuned; plain = BVH2 FP32 scene per soup, two launches "
                "per scene on one stream (ms includes launch gaps; kernel_sum excludes them)",
    }
    return out


# ---------------------------------------------------------------- quantised nodes

def to_original(hits, prim_indices):
    """Hit records (uint32 [n, 8]) with primId (a position in the tree's sorted
    order) replaced by the original triangle index, so that the hits of trees
    with different sorted orders compare."""
    h = np.array(hits, dtype=np.uint32, copy=True).reshape(-1, 8)
    m = h[:, 1] != 0xFFFFFFFF
    h[m, 1] = np.asarray(prim_indices, np.uint32)[h[m, 1]]
    return h


def hit_diff(hits, ref, name: str) -> dict:
    """Nearest-hit records (uint32 [n, 8]) against a reference set: mismatches
    (hit/miss differs, or t beyond 1e-5 relative: must be 0), ties resolved to
    another triangle (t within 1e-5 relative), and how many of those have the
    same t bit for bit."""
    diff = np.any(hits != ref, axis=1)
    hm = (hits[:, 3] != 0xFFFFFFFF) != (ref[:, 3] != 0xFFFFFFFF)
    tg = hits[:, 0].view(np.float32).astype(np.float64)
    tr = ref[:, 0].view(np.float32).astype(np.float64)
    near = np.abs(tg - tr) <= 1e-5 * np.abs(tr)
    return {f"nearest_mismatch_vs_{name}": int(np.count_nonzero(diff & (hm | ~near))),
            f"nearest_tie_vs_{name}": int(np.count_nonzero(diff & ~hm & near)),
            f"nearest_tie_exact_t_vs_{name}": int(np.count_nonzero(diff & ~hm & (hits[:, 0] == ref[:, 0])))}


def t_error_fp64(rays, hits, verts_all, sorted_idx_all, prim_base):
    """Relative error of the FP32 hit distance against the same ray-triangle
    intersection evaluated in FP64 (host), over the rays that hit."""
    h = hits.view(np.uint32).reshape(-1, 8)
    hit = h[:, 1] != 0xFFFFFFFF
    r = rays[hit].astype(np.float64)
    prim = h[hit, 1].astype(np.int64) + prim_base[h[hit, 3].astype(np.int64)]
    tri = sorted_idx_all.reshape(-1, 3)[prim].astype(np.int64)
    v = verts_all[:, :3].astype(np.float64)
    a, b, c = v[tri[:, 0]], v[tri[:, 1]], v[tri[:, 2]]
    o, d = r[:, 0:3], r[:, 4:7]
    e1, e2 = b - a, c - a
    pv = np.cross(d, e2)
    det = np.einsum("ij,ij->i", e1, pv)
    sv = o - a
    qv = np.cross(sv, e1)
    t64 = np.einsum("ij,ij->i", e2, qv) / det
    bu = np.einsum("ij,ij->i", sv, pv) / det
    bv = np.einsum("ij,ij->i", d, qv) / det
    t32 = h[hit, 0].view(np.float32).astype(np.float64)
    rel = np.abs(t32 - t64) / np.abs(t64)
    outside = int(np.count_nonzero((bu < -1e-6) | (bv < -1e-6) | (bu + bv > 1 + 1e-6)))
    return {"rays_checked": int(hit.sum()), "max_rel": float(rel.max()), "p99_rel": float(np.percentile(rel, 99)),
            "mean_rel": float(rel.mean()), "outside_fp64_triangle": outside}


def run_precision(ctx, args) -> dict:
    """Quantised-node precision, each scene traced separately as configured:
    the 2,097,152-triangle heightfield and the 8,388,608-triangle soup, each
    with 1920 x 1080 eye rays that all hit and 16 AO rays per hit (~33M).
    Every layout traces the same rays: the binary FP32 tree (the reference's
    decisions), BVH4 with FP32 boxes, FP16 boxes and 8-bit offsets.  Nearest
    hits of the quantised layouts are compared with the FP32-node build (same
    tree) and with the binary tree, any-hit flags with both, and the hit
    distance with an FP64 evaluation on 1M sampled eye rays per scene.  All of
    it twice: with the reference's Moller-Trumbore test, and with the FP32
    watertight test the configuration names (same rays)."""
    import torch

    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    layouts = [("bvh2", None), ("bvh4", 1), ("bvh4_f16", 1), ("bvh4_q8", 1)]
    res = {"note": "mismatch = hit/miss differs or t differs by more than 1e-5 relative (must be 0); tie = another "
                   "triangle at a t within 1e-5 relative (exact = the same t), resolved by visit order", "scenes": {}}

    def trace_layouts(w, d_eye, n_eye, tri_test, ao, d_ao):
        """Every layout with one triangle test; AO rays from the first
        (binary) layout's primary hits unless given.  Returns the layouts'
        entries, the AO rays (host, device) and the binary tree's FP64 t error."""
        out, ref_hits, ref_any, t_err = {}, None, None, None
        for layout, merge in layouts:
            sc = SceneRT(ctx, layout=layout, triangle_test=tri_test)
            if merge is not None:
                sc.set_bvh4_merge(merge)
            g = sc.AddGeom_Triangles3f(w.verts, len(w.verts), w.idx, w.idx.size, vByteStride=16)
            sc.AddInstance(g)
            sc.CommitScene()
            build_ms = sc.geom_info(g)["build_ms"]
            d_hits = torch.empty((n_eye, 8), dtype=torch.int32, device="cuda")
            sc.query_device(0, d_eye.data_ptr(), n_eye, d_hits.data_ptr(), sh)
            torch.cuda.synchronize()
            hits = d_hits.cpu().numpy().view(np.uint32)
            if t_err is None:
                si = sc.export(g, E.EXPORT_SORTED_INDICES)
                if ao is None:
                    ao = wl.frame_ao_rays(w, hits.view(np.float32), si)
                    d_ao = torch.from_numpy(ao).cuda()
                rng = np.random.default_rng(7)
                sample = np.sort(rng.choice(n_eye, size=min(1000000, n_eye), replace=False))
                t_err = t_error_fp64(w.eye_rays[sample], hits[sample], w.verts, si.astype(np.uint32),
                                     np.zeros(1, np.int64))
            n_ao = len(ao)
            d_any = torch.empty(n_ao, dtype=torch.uint8, device="cuda")
            for _ in range(3):
                sc.query_device(0, d_eye.data_ptr(), n_eye, d_hits.data_ptr(), sh)
                sc.query_device(1, d_ao.data_ptr(), n_ao, d_any.data_ptr(), sh)
            torch.cuda.synchronize()
            steps = 10
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            t_eye = t_ao = 0.0
            for _ in range(steps):
                e[0].record(stream)
                sc.query_device(0, d_eye.data_ptr(), n_eye, d_hits.data_ptr(), sh)
                e[1].record(stream)
                sc.query_device(1, d_ao.data_ptr(), n_ao, d_any.data_ptr(), sh)
                e[2].record(stream)
                torch.cuda.synchronize()
                t_eye += e[0].elapsed_time(e[1])
                t_ao += e[1].elapsed_time(e[2])
            t_eye /= steps
            t_ao /= steps
            anyf = d_any.cpu().numpy()
            pairs_eye, _ = sc.query_counters(0, d_eye.data_ptr(), n_eye, sh)
            pairs_ao, tris_ao = sc.query_counters(1, d_ao.data_ptr(), n_ao, sh)
            ao_bytes = LAYOUT_NODE_BYTES[layout] * pairs_ao + TRI_BYTES * tris_ao + (RAY_BYTES + 1) * n_ao
            pk, _ = measured_peak()
            entry = {"eye_ms": round(t_eye, 4), "ao_ms": round(t_ao, 4),
                     "mrays_s": round((n_eye + n_ao) / (t_eye + t_ao) / 1e3, 2), "build_ms": round(build_ms, 3),
                     "node_fetches_per_eye_ray": round(pairs_eye / n_eye, 3),
                     "node_fetches_per_ao_ray": round(pairs_ao / n_ao, 3),
                     "ao_roofline_frac": round(ao_bytes / (t_ao * 1e-3) / 1e9 / pk, 4),
                     "bvh_bytes": int(sc.geom_info(g)["bytes"])}
            if ref_hits is None:
                ref_hits, ref_any = hits, anyf
            else:
                entry.update(hit_diff(hits, ref_hits, "bvh2"))
                entry["anyhit_mismatch_vs_bvh2"] = int(np.count_nonzero(anyf != ref_any))
                if layout != "bvh4":
                    entry.update(hit_diff(hits, out["bvh4"]["_hits"], "fp32_nodes"))
                    entry["anyhit_mismatch_vs_fp32_nodes"] = int(np.count_nonzero(anyf != out["bvh4"]["_any"]))
            entry["_hits"] = hits
            entry["_any"] = anyf
            out[layout] = entry
            sc.close()
            del d_hits, d_any
        for k in out:
            out[k].pop("_hits")
            out[k].pop("_any")
        return out, ao, d_ao, t_err

    for scene_name in ("heightfield", "soup"):
        w = wl.config2(scene_name, args.width, args.height, args.soup_tris)
        d_eye = torch.from_numpy(w.eye_rays).cuda()
        n_eye = len(w.eye_rays)
        sc_res = {"workload": w.name, "tris": int(w.params["tris"])}
        out, ao, d_ao, t_err = trace_layouts(w, d_eye, n_eye, E.TRI_MOLLER_TRUMBORE, None, None)
        sc_res["t_error_vs_fp64"] = t_err
        sc_res["eye_rays"] = n_eye
        sc_res["ao_rays"] = int(len(ao))
        sc_res["layouts"] = out
        wt_out, _, _, wt_err = trace_layouts(w, d_eye, n_eye, E.TRI_WATERTIGHT, ao, d_ao)
        sc_res["watertight"] = {"t_error_vs_fp64": wt_err, "layouts": wt_out,
                                "note": "the same rays with the FP32 watertight test in every layout"}
        res["scenes"][scene_name] = sc_res
        del d_eye, d_ao
        torch.cuda.empty_cache()
    return res


def apply_frame(scene, args, collapse=True):
    """The headline scene's build options (before its first geometry): its
    Morton grid and, for 4-wide layouts, its collapse rule."""
    from heavyrt_gb300 import engine as E

    if args.morton_frame == "cubic":
        scene.set_morton_frame(E.MORTON_CUBIC)
    if collapse and args.bvh4_collapse == "largest_first":
        scene.set_bvh4_collapse(E.BVH4_COLLAPSE_LARGEST_FIRST)


def run_l2_window(scene, d_eye, d_ao, d_hits, d_any, args) -> dict:
    """The headline scene's eye and AO launches with a persisting-L2 window
    over its node array (hrt OPTION_L2_PERSIST) of 0 / 16 / 32 / 64 MiB set
    aside; results must equal the launches without a window."""
    import torch

    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    n_eye, n_ao = d_eye.shape[0], d_ao.shape[0]
    want_h, want_a = d_hits.clone(), d_any.clone()
    out = {"node_bytes": int(scene.export(0, 9).nbytes) if args.layout != "bvh2" else None, "sweep": []}
    steps = max(5, min(40, args.steps))
    for mib in (0, 16, 32, 64, 0):
        scene.set_l2_persist(mib)
        for _ in range(3):
            scene.query_device(0, d_eye.data_ptr(), n_eye, d_hits.data_ptr(), sh)
            scene.query_device(1, d_ao.data_ptr(), n_ao, d_any.data_ptr(), sh)
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record(stream)
        for _ in range(steps):
            scene.query_device(0, d_eye.data_ptr(), n_eye, d_hits.data_ptr(), sh)
        e[1].record(stream)
        for _ in range(steps):
            scene.query_device(1, d_ao.data_ptr(), n_ao, d_any.data_ptr(), sh)
        e[2].record(stream)
        torch.cuda.synchronize()
        out["sweep"].append({"mib": mib, "eye_ms": round(e[0].elapsed_time(e[1]) / steps, 4),
                             "ao_ms": round(e[1].elapsed_time(e[2]) / steps, 4),
                             "results_equal": bool(torch.equal(d_hits, want_h) and torch.equal(d_any, want_a))})
    scene.set_l2_persist(0)
    return out


def edge_distance64(rays, verts, sorted_idx, prim):
    """Smallest FP64 barycentric of each ray against the triangle at sorted
    position prim (negative: outside): the ray's distance to the triangle's
    nearest edge in barycentric units."""
    v = np.asarray(verts, np.float64)[:, :3]
    t = np.asarray(sorted_idx, np.int64).reshape(-1, 3)[np.asarray(prim, np.int64)]
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    o, d = rays[:, 0:3].astype(np.float64), rays[:, 4:7].astype(np.float64)
    e1, e2 = b - a, c - a
    pv = np.cross(d, e2)
    det = np.einsum("ij,ij->i", e1, pv)
    sv = o - a
    qv = np.cross(sv, e1)
    wb = np.einsum("ij,ij->i", sv, pv) / det
    wc = np.einsum("ij,ij->i", d, qv) / det
    return np.minimum(np.minimum(wb, wc), 1.0 - wb - wc)


def run_watertight(ctx, args, w, ao, mt_hits, mt_any, configs) -> dict:
    """The headline frame with the watertight triangle test (same layout,
    merge bound and launch shapes): its speed, and every ray whose result
    differs from the reference's MT test (hit/miss, or another triangle),
    classified by the ray's FP64 distance to the nearest edge of the triangle
    either test hit (barycentric units; MT accepts down to -1e-6)."""
    import torch

    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E

    sc = SceneRT(ctx, layout=args.layout, triangle_test=E.TRI_WATERTIGHT)
    if args.layout != "bvh2":
        sc.set_bvh4_merge(args.merge)
    apply_frame(sc, args)
    g = sc.AddGeom_Triangles3f(w.verts, w.verts.shape[0], w.idx, w.idx.size, vByteStride=16)
    sc.AddInstance(g)
    sc.CommitScene()
    for k in (0, 1):
        sc.set_trace_config(k, **configs[k])
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    n_eye, n_ao = len(w.eye_rays), len(ao)
    d_eye = torch.from_numpy(w.eye_rays).cuda()
    d_ao = torch.from_numpy(ao).cuda()
    d_hits = torch.empty((n_eye, 8), dtype=torch.int32, device="cuda")
    d_any = torch.empty(n_ao, dtype=torch.uint8, device="cuda")
    for _ in range(3):
        sc.query_device(0, d_eye.data_ptr(), n_eye, d_hits.data_ptr(), sh)
        sc.query_device(1, d_ao.data_ptr(), n_ao, d_any.data_ptr(), sh)
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    steps = max(5, min(50, args.steps))
    e[0].record(stream)
    for _ in range(steps):
        sc.query_device(0, d_eye.data_ptr(), n_eye, d_hits.data_ptr(), sh)
    e[1].record(stream)
    for _ in range(steps):
        sc.query_device(1, d_ao.data_ptr(), n_ao, d_any.data_ptr(), sh)
    e[2].record(stream)
    torch.cuda.synchronize()
    eye_ms, ao_ms = e[0].elapsed_time(e[1]) / steps, e[1].elapsed_time(e[2]) / steps
    si = sc.export(g, E.EXPORT_SORTED_INDICES)
    wt = d_hits.cpu().numpy().view(np.uint32)
    wt_any = d_any.cpu().numpy().astype(bool)
    sc.close()
    hm, hw = mt_hits[:, 3] != 0xFFFFFFFF, wt[:, 3] != 0xFFFFFFFF
    differ = (hm != hw) | (hm & hw & (mt_hits[:, 1] != wt[:, 1]))
    idx = np.nonzero(differ)[0]
    # FP64 smallest barycentric of the triangle each test hit (negative: the
    # ray passes outside that triangle)
    bm = np.full(idx.size, np.nan)
    bw = np.full(idx.size, np.nan)
    for hits, has, dst in ((mt_hits, hm, bm), (wt, hw, bw)):
        m = has[idx]
        if m.any():
            dst[m] = edge_distance64(w.eye_rays[idx[m]], w.verts, si, hits[idx[m], 1])
    slack = 1e-6  # the reference test's own barycentric slack
    classes = {
        # the reference's MT accepted a triangle the ray passes outside of, beyond its slack
        "mt_hit_outside_beyond_slack": int(np.count_nonzero(bm < -slack)),
        # the reference's MT missed while the ray passes inside the triangle the watertight test hit (a leak)
        "mt_miss_inside": int(np.count_nonzero(~hm[idx] & (bw > 0))),
        # the watertight test hit a triangle the FP64 ray passes outside of (its FP32 projection)
        "wt_hit_outside_beyond_slack": int(np.count_nonzero(bw < -slack)),
        # both within the slack of a shared edge: another of the triangles meeting there
        "edge_ties": int(np.count_nonzero(((np.abs(bm) <= slack) | np.isnan(bm)) & ((np.abs(bw) <= slack) | np.isnan(bw)))),
    }
    depth = {"mt_outside_max": float(-np.nanmin(bm)) if np.any(bm < -slack) else 0.0,
             "mt_leak_inside_max": float(np.nanmax(np.where(~hm[idx], bw, np.nan))) if np.any(~hm[idx] & (bw > 0))
             else 0.0,
             "wt_outside_max": float(-np.nanmin(bw)) if np.any(bw < -slack) else 0.0}
    same = hm & hw & (mt_hits[:, 1] == wt[:, 1])
    tm = mt_hits[same, 0].view(np.float32).astype(np.float64)
    tw = wt[same, 0].view(np.float32).astype(np.float64)
    return {"layout": args.layout, "eye_ms": round(eye_ms, 4), "ao_ms": round(ao_ms, 4),
            "mrays_s": round((n_eye + n_ao) / (eye_ms + ao_ms) / 1e3, 2),
            "eye_rays_differing_from_mt": int(idx.size), "eye_hits_mt": int(hm.sum()), "eye_hits_wt": int(hw.sum()),
            "differing_by_class": classes, "barycentric_depth": depth,
            "same_triangle_t_max_rel_vs_mt": float((np.abs(tm - tw) / np.abs(tm)).max()) if tm.size else 0.0,
            "ao_rays_differing_from_mt": int(np.count_nonzero(wt_any != mt_any)),
            "note": "barycentric = smallest FP64 barycentric of the ray against the triangle a test hit "
                    "(negative: outside); MT accepts down to -1e-6"}


# ---------------------------------------------------------------- served stream

def served_workload(args, rate: float, seconds: float):
    """64 resident scenes, the arrival trace, ray pools and upload scenes."""
    from heavyrt_gb300 import workload as wl

    seed = 0x5EED0005
    n_tris = wl.log_uniform_counts(seed, 1, 64, 10000, 2000000)
    scenes = []
    for i, n in enumerate(n_tris):
        if i % 2 == 0:
            scenes.append(wl.soup(seed + 100 + i, int(n), -1.0, 1.0, 0.02))
        else:
            side = max(2, int(round((int(n) / 2) ** 0.5)))
            v, idx, _ = wl.heightfield(seed + 100 + i, side, side)
            scenes.append((v, idx))
    up_tris = wl.log_uniform_counts(seed, 2, 6, 100000, 1000000)
    uploads = [wl.soup(seed + 300 + i, int(n), -1.0, 1.0, 0.02) for i, n in enumerate(up_tris)]
    rng = np.random.default_rng(seed)
    count = int(rate * seconds)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    sizes = wl.log_uniform_counts(seed, 3, count, 1000, 1000000)
    target = rng.integers(0, len(scenes), count)
    kinds = rng.integers(0, 2, count)
    upload = rng.random(count) < 0.05
    pools = [wl.sphere_rays(seed + 400 + k, 1000000, 3.0) for k in range(4)]
    return {"scenes": scenes, "uploads": uploads, "arrivals": arrivals, "sizes": sizes, "target": target,
            "kinds": kinds, "upload": upload, "pools": pools,
            "tris": [int(len(x[1]) // 3) for x in scenes]}


def _class_stats(lat_s, upload, sizes):
    """p50/p99 of ray-only requests, of requests of at least 256k rays, and of uploads."""
    lat = np.asarray(lat_s) * 1e3
    out = {}
    for name, m in (("rays_only", ~upload), ("rays_only_256k_plus", ~upload & (sizes >= 262144)), ("uploads", upload)):
        if m.any():
            out[f"{name}_p50_ms"] = round(float(np.percentile(lat[m], 50)), 3)
            out[f"{name}_p99_ms"] = round(float(np.percentile(lat[m], 99)), 3)
    return out


def _latency_stats(lat_s, rays, span_s):
    lat = np.sort(np.asarray(lat_s)) * 1e3
    return {"p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
            "max_ms": round(float(lat[-1]), 3), "mrays_s": round(rays / span_s / 1e6, 2),
            "requests": int(len(lat))}


def torch_device() -> int:
    import torch

    return torch.cuda.current_device()


def run_served(ctx, args, rate: float = None, seconds: float = None) -> dict:
    """Served stream: 64 resident scenes (soups and heightfields, log-uniform
    10k..2M triangles), Poisson arrivals, each request log-uniform 1k..1M rays
    against a uniformly chosen scene, half nearest / half any; 5% of requests
    upload a new 100k..1M-triangle scene (built on arrival, evictable) and
    query it.  "served": the engine's server (continuous batching over
    resident scenes, 150 GB budget); "plain": the same arrivals handled one at
    a time in arrival order through the host-pointer query of one BVH2 scene
    per geometry.  Latency = completion - scheduled arrival."""
    import queue as Q

    from heavyrt_gb300 import PinnedBuffer, SceneRT
    from heavyrt_gb300 import engine as E

    rate = args.served_rate if rate is None else rate
    seconds = args.served_seconds if seconds is None else seconds
    W = served_workload(args, rate, seconds)
    arrivals, sizes, target, kinds, upload = W["arrivals"], W["sizes"], W["target"], W["kinds"], W["upload"]
    count = len(arrivals)
    pools = []
    for p in W["pools"]:
        b = PinnedBuffer(p.nbytes)
        b.array(np.float32).reshape(-1, 8)[:] = p
        pools.append(b)
    ring = 64
    outs = [PinnedBuffer(32 * 1000000) for _ in range(ring)]
    # upload meshes in page-locked memory, as a serving client holds its inputs
    up_bufs = []
    for v, idx in W["uploads"]:
        bv, bi = PinnedBuffer(v.nbytes), PinnedBuffer(idx.nbytes)
        av = bv.array(np.float32).reshape(v.shape)
        ai = bi.array(np.uint32)
        av[:] = v
        ai[:] = idx
        up_bufs.append((bv, bi, av, ai))
    W["uploads"] = [(av, ai) for _, _, av, ai in up_bufs]
    result = {"workload": f"served: 64 resident scenes ({sum(W['tris'])} tris), Poisson {rate:.0f} req/s "
                          f"for {seconds:.1f} s, 1k..1M rays per request, 5% uploads",
              "requests": count, "rays": int(sizes.sum()), "uploads": int(upload.sum())}

    # ---- served
    # the headline's Morton grid for every scene the server builds (free at
    # build time); the even-depth collapse, since the largest-first roles'
    # level launches add ~0.15 ms to each upload (upload p50 1.24 -> 1.42 ms)
    # while saving only a few percent of these requests' short traversals
    srv = E.Server(ctx, memory_budget=150 * 10**9, layout="bvh4_f16", bvh4_merge=1,
                   morton_frame=E.MORTON_CUBIC if args.morton_frame == "cubic" else E.MORTON_PER_AXIS,
                   bvh4_collapse=E.BVH4_COLLAPSE_EVEN_DEPTH)
    t0 = time.perf_counter()
    ids = [srv.add_scene(v, idx, evictable=False) for v, idx in W["scenes"]]
    for i in ids:
        assert srv.scene_state(i, timeout=600) == E.SCENE_READY
    setup_s = time.perf_counter() - t0
    lat = np.zeros(count)
    lat_engine = np.zeros(count)  # submission to completion, as the server records them
    tickets = Q.Queue()
    busy = [False] * ring  # output buffer in use by a request in flight
    done_lock = threading.Condition()
    up_q = Q.Queue()
    infos = [None] * count

    def waiter():
        while True:
            item = tickets.get()
            if item is None:
                return
            j, t, lag = item
            st, info = srv.wait(t)
            if st != 0:
                raise RuntimeError(f"served request {j} failed: {st}")
            lat_engine[j] = info["tDone"] - info["tSubmit"]
            lat[j] = lat_engine[j] + lag
            infos[j] = info
            with done_lock:
                busy[j % ring] = False
                done_lock.notify_all()

    def submit(j, sid, start):
        with done_lock:
            while busy[j % ring]:
                done_lock.wait()
            busy[j % ring] = True
        n = int(sizes[j])
        t = srv.submit(sid, int(kinds[j]), pools[j % 4].ptr, n, outs[j % ring].ptr)
        tickets.put((j, t, time.perf_counter() - start - arrivals[j]))

    def uploader(start):
        while True:
            j = up_q.get()
            if j is None:
                return
            v, idx = W["uploads"][j % len(W["uploads"])]
            sid = srv.add_scene(v, idx, evictable=True)
            submit(j, sid, start)

    wt = threading.Thread(target=waiter)
    wt.start()
    clk = ClockSampler(torch_device())
    clk.start()
    start = time.perf_counter()
    ut = threading.Thread(target=uploader, args=(start,))
    ut.start()
    for j in range(count):
        d = start + arrivals[j] - time.perf_counter()
        if d > 0:
            time.sleep(d)
        if upload[j]:
            up_q.put(j)
        else:
            submit(j, ids[int(target[j])], start)
    up_q.put(None)
    ut.join()
    tickets.put(None)
    wt.join()
    span = time.perf_counter() - start
    clk.stop()
    served_clocks = clk.spread()
    st = srv.stats()
    srv.close()
    served = _latency_stats(lat, float(sizes.sum()), span)
    served.update(_class_stats(lat, upload, sizes))
    bsz = [i["batchRequests"] for i in infos]
    served.update({"batches": int(st["batches"]), "mean_requests_per_batch": round(float(np.mean(bsz)), 2),
                   "max_requests_per_batch": int(max(bsz)), "builds": int(st["builds"]),
                   "evictions": int(st["evictions"]), "peak_resident_gb": round(st["peakResidentBytes"] / 1e9, 2),
                   "upload_p50_ms": round(float(np.percentile(lat[upload] * 1e3, 50)), 3) if upload.any() else None,
                   "setup_s": round(setup_s, 2), "layout": "bvh4_f16 (merge 1)",
                   "engine_p50_ms": round(float(np.percentile(lat_engine * 1e3, 50)), 3),
                   "engine_p99_ms": round(float(np.percentile(lat_engine * 1e3, 99)), 3),
                   "client_lag_p99_ms": round(float(np.percentile((lat - lat_engine) * 1e3, 99)), 3),
                   "queued_p99_ms": round(float(np.percentile([(i["tStart"] - i["tSubmit"]) * 1e3 for i in infos], 99)), 3),
                   "batch_p99_ms": round(float(np.percentile([(i["tDone"] - i["tStart"]) * 1e3 for i in infos], 99)), 3)})

    # ---- plain: one request at a time, in arrival order
    plain_scenes = []
    for v, idx in W["scenes"]:
        sc = SceneRT(ctx)
        g = sc.AddGeom_Triangles3f(v, len(v), idx, idx.size, vByteStride=16)
        sc.AddInstance(g)
        sc.CommitScene()
        plain_scenes.append(sc)
    L = E.lib()
    import ctypes as C

    lat_p = np.zeros(count)
    clk = ClockSampler(torch_device())
    clk.start()
    start = time.perf_counter()
    for j in range(count):
        d = start + arrivals[j] - time.perf_counter()
        if d > 0:
            time.sleep(d)
        n = int(sizes[j])
        if upload[j]:
            v, idx = W["uploads"][j % len(W["uploads"])]
            sc = SceneRT(ctx)
            g = sc.AddGeom_Triangles3f(v, len(v), idx, idx.size, vByteStride=16)
            sc.AddInstance(g)
            sc.CommitScene()
        else:
            sc = plain_scenes[int(target[j])]
        f = L.hrt_query_nearest_host if kinds[j] == 0 else L.hrt_query_any_host
        ctx.check(f(sc._h, C.c_void_p(pools[j % 4].ptr), n, C.c_void_p(outs[0].ptr)), "plain query")
        if upload[j]:
            sc.close()
        lat_p[j] = time.perf_counter() - start - arrivals[j]
    span_p = time.perf_counter() - start
    clk.stop()
    plain_clocks = clk.spread()
    for sc in plain_scenes:
        sc.close()
    W["uploads"] = None
    for b in pools + outs + [x for bv, bi, _, _ in up_bufs for x in (bv, bi)]:
        b.free()
    result["served"] = served
    result["plain"] = _latency_stats(lat_p, float(sizes.sum()), span_p)
    result["plain"].update(_class_stats(lat_p, upload, sizes))
    result["plain"]["layout"] = "bvh2"
    result["served"]["clocks"] = served_clocks
    result["plain"]["clocks"] = plain_clocks
    result["note"] = ("Mrays/s = rays of all requests / (last completion - first arrival): at an offered load below "
                      "capacity it equals the offered rate; the latencies show the difference")
    return result


# ---------------------------------------------------------------- GPU engine

def run_builds(ctx, args, w):
    """K builds of the headline scene; GPU build time of each (CUDA events around the build's launches)."""
    from heavyrt_gb300 import SceneRT

    ms = []
    for _ in range(args.only_build):
        s = SceneRT(ctx, layout=args.layout)
        if args.layout != "bvh2":
            s.set_bvh4_merge(args.merge)
        apply_frame(s, args)
        g = s.AddGeom_Triangles3f(w.verts, w.verts.shape[0], w.idx, w.idx.size, vByteStride=16)
        s.AddInstance(g)
        s.CommitScene()
        ms.append(s.geom_info(g)["build_ms"])
        s.close()
    return {"workload": f"heightfield{args.nx}x{args.nx} ({w.idx.size // 3} tris), {args.layout} (merge {args.merge})",
            "builds": len(ms), "build_ms": [round(x, 4) for x in ms],
            "median_ms": round(statistics.median(ms), 4) if ms else None}


def run_builds_batched(ctx, args):
    """K segmented builds of the 256-soup batch (BVH4 FP16, merge 1); GPU build time of each."""
    from heavyrt_gb300 import autotune as AT
    from heavyrt_gb300 import workload as wl

    w = wl.config3(args.batch_scenes)
    ms = []
    for _ in range(args.only_build_batched):
        scene, ids = AT.build_batch(ctx, w.verts, w.idx, "bvh4_f16", 1)
        ms.append(scene.geom_info(ids[0])["build_ms"])
        scene.close()
    return {"workload": f"soups{len(w.verts)} ({sum(int(i.size) // 3 for i in w.idx)} tris), bvh4_f16 (merge 1)",
            "builds": len(ms), "build_ms": [round(x, 4) for x in ms],
            "median_ms": round(statistics.median(ms), 4) if ms else None}


def run_frames(ctx, args, w, trace_configs=None) -> dict:
    """Whole frames of HeavyRT's two example renderers on the device (hrt_frame):
    RTAO (examples/02_rtao: eye rays, nearest hit, hit shading, 16 AO rays per
    hit pixel from the renderer's quasi-random tile, any-hit, AO2Color) and the
    eye-ray renderer (examples/01_eye_rays: packed pixel order, nearest hit,
    palette), on the heightfield scene, timed frame to frame."""
    import torch

    from heavyrt_gb300 import Frame, SceneRT, rtao_qmc_tile
    from heavyrt_gb300 import workload as wl

    W, H, R = args.width, args.height, 16
    sc = SceneRT(ctx, layout=args.layout)
    if args.layout != "bvh2":
        sc.set_bvh4_merge(args.merge)
    apply_frame(sc, args)
    g = sc.AddGeom_Triangles3f(w.verts, w.verts.shape[0], w.idx, w.idx.size, vByteStride=16)
    sc.AddInstance(g)
    sc.CommitScene()
    for kind, cfg in (trace_configs or {}).items():
        # the frames trace their eye rays in the renderer's own packed order
        sc.set_trace_config(kind, **dict(cfg, imageWidth=0))
    f = Frame(ctx)
    f.set_normals(g, wl.vertex_normals(w.verts, w.idx))
    f.set_ao_tile(rtao_qmc_tile(R), R)
    p, v = wl.camera_inverses((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, W, H)
    radius = float(w.params["ao_length"])
    colors = torch.empty(W * H, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream()
    frames = max(10, min(100, args.steps // 3))

    def timed(render):
        for _ in range(3):
            render()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(frames):
            render()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / frames

    def rtao():
        f.render_rtao(sc, p, v, W, H, colors.data_ptr(), 0.0, 3.4028234663852886e38, radius, 1.0,
                      stream=st.cuda_stream)

    def eye():
        f.render_eye(sc, p, v, W, H, colors.data_ptr(), stream=st.cuda_stream)

    ms_rtao = timed(rtao)
    from heavyrt_gb300 import engine as E

    slots = f.buffer(E.FRAME_AO_PIXEL)[1]
    n_ao = f.buffer(E.FRAME_AO_RAYS)[1]
    lit = colors.cpu().numpy().view(np.uint32)
    ms_eye = timed(eye)
    out = {"workload": f"{W}x{H} frames of the example renderers on heightfield{args.nx}x{args.nx} "
                       f"({w.idx.size // 3} tris), {args.layout} (merge {args.merge})",
           "rtao": {"ms_per_frame": round(ms_rtao, 4), "eye_rays": W * H, "hit_pixels": int(slots),
                    "ao_rays": int(n_ao), "ao_rays_per_hit_pixel": R, "ao_max_radius": round(radius, 5),
                    "mrays_s": round((W * H + n_ao) / (ms_rtao * 1e3), 2),
                    "frames_per_s": round(1e3 / ms_rtao, 1),
                    "mean_gray_of_hit_pixels": round(float((lit[lit != 0] & 0xFF).mean()) if (lit != 0).any() else 0.0, 2),
                    "device_syncs_per_frame": 1},
           "eye": {"ms_per_frame": round(ms_eye, 4), "mrays_s": round(W * H / (ms_eye * 1e3), 2),
                   "frames_per_s": round(1e3 / ms_eye, 1)},
           "frames_timed": frames}
    f.close()
    sc.close()
    return out


def run_engine(args):
    import torch

    from heavyrt_gb300 import replicas

    rk = replicas.from_env()
    rank, world, local = rk.rank, rk.world, rk.local
    torch.cuda.set_device(local)
    replicas.init(rk, "nccl")
    from heavyrt_gb300 import Context, PinnedBuffer, SceneRT
    from heavyrt_gb300 import engine as E

    ctx = Context(local)
    if args.only_build_batched:
        if rank == 0:
            print(json.dumps({"build_batched": run_builds_batched(ctx, args)}), flush=True)
        return 0
    if args.only_batched:
        if rank == 0:
            print(json.dumps({"batched": run_batched(ctx, args)}), flush=True)
        return 0
    if args.only_served:
        if rank == 0:
            print(json.dumps({"served": run_served(ctx, args)}), flush=True)
        return 0
    if args.only_precision:
        if rank == 0:
            print(json.dumps({"precision": run_precision(ctx, args)}), flush=True)
        return 0
    w = make_frame(args)
    if args.only_build:
        if rank == 0:
            print(json.dumps({"build": run_builds(ctx, args, w)}), flush=True)
        return 0
    if args.only_frames:
        if rank == 0:
            print(json.dumps({"frames": run_frames(ctx, args, w)}), flush=True)
        return 0

    def make_scene(layout, frame=True, collapse=True):
        sc = SceneRT(ctx, layout=layout)
        if layout != "bvh2":
            sc.set_bvh4_merge(args.merge)
        if frame:
            apply_frame(sc, args, collapse)
        elif collapse and args.bvh4_collapse == "largest_first":
            sc.set_bvh4_collapse(E.BVH4_COLLAPSE_LARGEST_FIRST)
        g = sc.AddGeom_Triangles3f(w.verts, w.verts.shape[0], w.idx, w.idx.size, vByteStride=16)
        sc.AddInstance(g)
        sc.CommitScene()
        return sc, g

    scene, gid = make_scene(args.layout)
    prim_idx = scene.export(gid, E.EXPORT_PRIM_INDICES)
    if args.l2_persist:
        scene.set_l2_persist(args.l2_persist)
    info = scene.geom_info(gid)
    # build time: a few more builds of the same geometry
    build_ms = [info["build_ms"]]
    for _ in range(0 if args.ncu else 3):
        s2, g2 = make_scene(args.layout)
        build_ms.append(s2.geom_info(g2)["build_ms"])
        s2.close()

    eye_hits = scene.RayQuery_NearestHit(w.eye_rays)
    ao = ao_from_hits(w, eye_hits, scene.export(gid, E.EXPORT_SORTED_INDICES))
    frame_eye, frame_ao = w.eye_rays, ao
    frame_rays = frame_eye.shape[0] + frame_ao.shape[0]
    split = args.split == "rays" and world > 1
    if split:
        # this rank's share of the frame: whole 8-row bands of the image (the
        # tile order stays within the share) and a run of AO rays
        e0, e1 = replicas.partition(frame_eye.shape[0], rk, align=8 * args.width)
        a0, a1 = replicas.partition(frame_ao.shape[0], rk, align=16)
        w.eye_rays = np.ascontiguousarray(frame_eye[e0:e1])
        ao = np.ascontiguousarray(frame_ao[a0:a1])
        # sections that make or trace whole frames of their own stay out
        args.no_frames = args.no_watertight = args.no_l2_sweep = args.no_frame_compare = args.no_plain = True
        args.no_served = args.no_batched = args.no_precision = True
    n_eye, n_ao = w.eye_rays.shape[0], ao.shape[0]

    def job_rate(local_units, ms):
        """Whole-job units per second: the frame over the slowest rank's time
        when the ranks split it, every replica's units otherwise."""
        return frame_rays / (ms * 1e-3) if split else replicas.job_throughput(rk, local_units, ms)

    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    d_eye = torch.from_numpy(w.eye_rays).cuda()
    d_ao = torch.from_numpy(ao).cuda()
    d_hits = torch.empty((n_eye, 8), dtype=torch.int32, device="cuda")
    d_any = torch.empty(n_ao, dtype=torch.uint8, device="cuda")

    # algorithmic bytes per launch from the counting traversal (same decisions)
    if args.ncu:
        eye_pairs = eye_tris = ao_pairs = ao_tris = 0
    else:
        eye_pairs, eye_tris = scene.query_counters(0, d_eye.data_ptr(), n_eye, sh)
        ao_pairs, ao_tris = scene.query_counters(1, d_ao.data_ptr(), n_ao, sh)
    node_bytes = LAYOUT_NODE_BYTES[args.layout]
    eye_bytes = node_bytes * eye_pairs + TRI_BYTES * eye_tris + RAY_BYTES * n_eye + 32 * n_eye
    ao_bytes = node_bytes * ao_pairs + TRI_BYTES * ao_tris + RAY_BYTES * n_ao + 1 * n_ao

    # the eye rays are one row-major image: let the traversal take them in
    # 4 x 8 pixel tiles (the autotuner keeps this property of the rays)
    if args.eye_order == "tiles":
        scene.set_trace_config(0, imageWidth=args.width)
    tuned = None
    fixed = {0: args.launch_nearest, 1: args.launch_any}
    if any(fixed.values()) or (not args.no_autotune and not args.ncu):
        tuned = {}
        for kind, (dr, n, do) in enumerate(((d_eye, n_eye, d_hits), (d_ao, n_ao, d_any))):
            if fixed[kind]:
                vals = [int(x) for x in fixed[kind].split(",")]
                cfg = dict(zip(["threadsPerBlock", "persistent", "stepsPerRefill", "refillLanes", "stackEntries"],
                               vals))
                cfg["imageWidth"] = scene.trace_config(kind)["imageWidth"]
                scene.set_trace_config(kind, **cfg)
                tuned[kind] = scene.trace_config(kind)
            elif not args.no_autotune and not args.ncu:
                tuned[kind], _ = scene.autotune(E.query_desc(kind, dr.data_ptr(), n, do.data_ptr()), 3)

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        scene.query_device(0, d_eye.data_ptr(), n_eye, d_hits.data_ptr(), sh)
        if ev:
            ev[1].record(stream)
        scene.query_device(1, d_ao.data_ptr(), n_ao, d_any.data_ptr(), sh)
        if ev:
            ev[2].record(stream)

    for _ in range(args.warmup if args.ncu else max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    replicas.barrier(rk)
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        step(evs[k])
    t_end.record(stream)
    torch.cuda.synchronize()
    replicas.barrier(rk)
    clk = clocks.stop()
    total_ms = t_start.elapsed_time(t_end)
    eye_ms = [e[0].elapsed_time(e[1]) for e in evs]
    ao_ms = [e[1].elapsed_time(e[2]) for e in evs]
    total_ms = replicas.max_over_ranks(rk, total_ms, "cuda")  # the slowest replica's time
    ms_per_step = total_ms / args.steps
    rays_per_step = n_eye + n_ao
    value = job_rate(rays_per_step, ms_per_step) / 1e6
    if args.ncu:
        print(json.dumps({"ncu_run": True, "ms_per_step": ms_per_step, "value": value}), flush=True)
        return 0

    # e2e: host pinned rays in, results out, through the host-pointer C-ABI calls
    pin_eye = PinnedBuffer(w.eye_rays.nbytes)
    pin_ao = PinnedBuffer(ao.nbytes)
    pin_hits = PinnedBuffer(32 * n_eye)
    pin_any = PinnedBuffer(n_ao)
    pe = pin_eye.array(np.float32).reshape(-1, 8)
    pa = pin_ao.array(np.float32).reshape(-1, 8)
    pe[:] = w.eye_rays
    pa[:] = ao
    L = E.lib()
    import ctypes as C

    def e2e_step_sync():
        ctx.check(L.hrt_query_nearest_host(scene._h, C.c_void_p(pin_eye.ptr), n_eye, C.c_void_p(pin_hits.ptr)), "e2e")
        ctx.check(L.hrt_query_any_host(scene._h, C.c_void_p(pin_ao.ptr), n_ao, C.c_void_p(pin_any.ptr)), "e2e")

    # the same two batches enqueued on two streams (reported beside the value):
    # both streams are waited for, then the scene's device-side checks read
    s_eye, s_ao = torch.cuda.Stream(), torch.cuda.Stream()

    def e2e_step():
        ctx.check(L.hrt_query_nearest_host_async(scene._h, C.c_void_p(pin_eye.ptr), n_eye, C.c_void_p(pin_hits.ptr),
                                                 C.c_void_p(s_eye.cuda_stream)), "e2e")
        ctx.check(L.hrt_query_any_host_async(scene._h, C.c_void_p(pin_ao.ptr), n_ao, C.c_void_p(pin_any.ptr),
                                             C.c_void_p(s_ao.cuda_stream)), "e2e")
        s_eye.synchronize()
        s_ao.synchronize()
        ctx.check(L.hrt_scene_check(scene._h), "e2e")

    def time_steps(fn):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fn()
        return replicas.max_over_ranks(rk, (time.perf_counter() - t0) / args.steps, "cuda")

    e2e_async_s = time_steps(e2e_step)
    e2e_s = time_steps(e2e_step_sync)
    e2e_value = job_rate(rays_per_step, 1e3 * e2e_s) / 1e6
    e2e_async_value = job_rate(rays_per_step, 1e3 * e2e_async_s) / 1e6
    # the two calls of the synchronous step timed on their own (wall clock)
    e2e_eye_s = time_steps(lambda: ctx.check(L.hrt_query_nearest_host(scene._h, C.c_void_p(pin_eye.ptr), n_eye,
                                                                      C.c_void_p(pin_hits.ptr)), "e2e"))
    e2e_ao_s = time_steps(lambda: ctx.check(L.hrt_query_any_host(scene._h, C.c_void_p(pin_ao.ptr), n_ao,
                                                                 C.c_void_p(pin_any.ptr)), "e2e"))
    got_any = pin_any.array(np.uint8)[:n_ao].copy()

    # split frame: every rank's results gathered on rank 0 through host
    # memory (after the timed region) and compared with rank 0 tracing the
    # whole frame itself
    split_check = None
    if split:
        grp = replicas.host_group(rk)
        all_hits = replicas.gather_rows(rk, d_hits.cpu().numpy().view(np.uint32), grp)
        all_any = replicas.gather_rows(rk, got_any, grp)
        if rank == 0:
            f_hits = scene.RayQuery_NearestHit(frame_eye).view(np.uint32).reshape(-1, 8)
            f_any = scene.RayQuery_AnyHit(frame_ao).astype(np.uint8)
            split_check = {"ranks": world, "gathered_rays": int(all_hits.shape[0] + all_any.shape[0]),
                           "frame_rays": int(frame_rays),
                           "nearest_mismatch": int(np.count_nonzero(np.any(all_hits != f_hits, axis=1))),
                           "anyhit_mismatch": int(np.count_nonzero(all_any != f_any))}

    raygen_e2e = None
    if not split:
        # the same frame with its rays made on the device: camera parameters in,
        # eye hits and AO flags out (no ray crosses the host link)
        pp = w.params
        cap = n_eye * pp["ao_per_hit"]
        g_eye = torch.empty((n_eye, 8), dtype=torch.float32, device="cuda")
        g_hits = torch.empty((n_eye, 8), dtype=torch.int32, device="cuda")
        g_ao = torch.empty((cap, 8), dtype=torch.float32, device="cuda")
        g_any = torch.empty(cap, dtype=torch.uint8, device="cuda")

        copy_stream = torch.cuda.Stream()
        eye_done = torch.cuda.Event()

        def raygen_step():
            # the eye hits go home on a second stream while the AO rays are made
            # and traced; the AO flags are written straight into page-locked host memory
            ctx.gen_pinhole_rays((0.0, -2.5, 1.5), (0, 0, 0), (0, 0, 1), 60.0, args.width, args.height, 0.0, 1e9,
                                 g_eye.data_ptr(), sh)
            scene.query_device(0, g_eye.data_ptr(), n_eye, g_hits.data_ptr(), sh)
            eye_done.record(stream)
            copy_stream.wait_event(eye_done)
            with torch.cuda.stream(copy_stream):
                pin_hits_d.copy_(g_hits, non_blocking=True)
            k = scene.gen_ao_rays(pp["ao_seed"], g_eye.data_ptr(), g_hits.data_ptr(), n_eye, pp["ao_per_hit"],
                                  pp["ao_length"], pp["ao_offset"], g_ao.data_ptr(), cap, 0, sh)
            scene.query_device(1, g_ao.data_ptr(), k, pin_any_d.data_ptr(), sh)
            torch.cuda.synchronize()
            return k

        pin_hits_d = torch.empty((n_eye, 8), dtype=torch.int32).pin_memory()
        pin_any_d = torch.empty(cap, dtype=torch.uint8).pin_memory()
        for _ in range(3):
            n_ao_dev = raygen_step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            n_ao_dev = raygen_step()
        rg_s = replicas.max_over_ranks(rk, (time.perf_counter() - t0) / args.steps, "cuda")
        raygen_e2e = {"value": round(replicas.job_throughput(rk, n_eye + n_ao_dev, 1e3 * rg_s) / 1e6, 3), "unit": UNIT,
                      "h2d_bytes_per_step": 0, "d2h_bytes_per_step": int(32 * n_eye + n_ao_dev),
                      "ao_rays": int(n_ao_dev), "ao_rays_equal_host_count": bool(n_ao_dev == n_ao),
                      "anyhit_equal_host_frame": bool(np.array_equal(pin_any_d[:n_ao_dev].numpy(), got_any))
                      if n_ao_dev == n_ao else False}
        del g_eye, g_hits, g_ao, g_any
    for b in (pin_eye, pin_ao, pin_hits, pin_any):
        b.free()
    if split:
        raygen_e2e = {"skipped": "the ranks split the frame's rays; device ray generation makes whole frames"}

    # the persisting-L2 set-aside ends with the headline scene's legs (the
    # other sections run without it)
    if args.l2_persist:
        scene.set_l2_persist(0)
    # plain: the binary FP32 tree (the reference's decisions) with the default launch shape
    plain = None
    if not args.no_plain:
        ps, _ = make_scene("bvh2", frame=False)  # the reference's grid and decisions
        p_hits = torch.empty_like(d_hits)
        p_any = torch.empty_like(d_any)
        for _ in range(3):
            ps.query_device(0, d_eye.data_ptr(), n_eye, p_hits.data_ptr(), sh)
            ps.query_device(1, d_ao.data_ptr(), n_ao, p_any.data_ptr(), sh)
        torch.cuda.synchronize()
        pe = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
        for k in range(args.steps):
            pe[k][0].record(stream)
            ps.query_device(0, d_eye.data_ptr(), n_eye, p_hits.data_ptr(), sh)
            pe[k][1].record(stream)
            ps.query_device(1, d_ao.data_ptr(), n_ao, p_any.data_ptr(), sh)
            pe[k][2].record(stream)
        torch.cuda.synchronize()
        pe_ms = statistics.mean(e[0].elapsed_time(e[1]) for e in pe)
        pa_ms = statistics.mean(e[1].elapsed_time(e[2]) for e in pe)
        hp = to_original(p_hits.cpu().numpy().view(np.uint32), ps.export(0, E.EXPORT_PRIM_INDICES))
        hq = to_original(d_hits.cpu().numpy().view(np.uint32), prim_idx)
        plain = {"layout": LAYOUT_DESC["bvh2"], "eye_ms": round(pe_ms, 4), "ao_ms": round(pa_ms, 4),
                 "mrays_s": round((n_eye + n_ao) / (pe_ms + pa_ms) / 1e3, 2),
                 **hit_diff(hq, hp, "plain"),
                 "anyhit_mismatch": int(np.count_nonzero(p_any.cpu().numpy() != d_any.cpu().numpy()))}
        if not args.ncu:
            pp_eye, pt_eye = ps.query_counters(0, d_eye.data_ptr(), n_eye, sh)
            p_bytes = 64 * pp_eye + TRI_BYTES * pt_eye + RAY_BYTES * n_eye + 32 * n_eye
            p_ach = p_bytes / (pe_ms * 1e-3) / 1e9
            pk, _ = measured_peak()
            plain["coherent_eye_roofline"] = {"achieved": round(p_ach, 1), "frac": round(p_ach / pk, 4),
                                              "algorithmic_bytes_per_launch": int(p_bytes),
                                              "node_pairs_per_eye_ray": round(pp_eye / n_eye, 3)}
            # HeavyRT's own bytes-loaded accounting (m_stats.BLB, core/BVH2CommonRT.cpp:68-70,125:
            # 2 x 32 B per node step, 3 x 4 B + 3 x 16 B per tested triangle) on the same rays, with
            # the BVH2 kernel's counts (the decisions of BVH2TraverseC32) and nearest-hit traversal
            # for the AO rays too, the way the reference answers any-hit
            pp_ao, pt_ao = ps.query_counters(0, d_ao.data_ptr(), n_ao, sh)
            blb_eye = (64 * pp_eye + 60 * pt_eye) / n_eye
            blb_ao = (64 * pp_ao + 60 * pt_ao) / n_ao
            plain["reference_blb"] = {
                "eye_bytes_per_ray": round(blb_eye, 2), "ao_bytes_per_ray": round(blb_ao, 2),
                "eye_node_pairs_per_ray": round(pp_eye / n_eye, 3), "eye_tris_per_ray": round(pt_eye / n_eye, 3),
                "ao_node_pairs_per_ray": round(pp_ao / n_ao, 3), "ao_tris_per_ray": round(pt_ao / n_ao, 3),
                "at_plain_rate_gb_s": round((blb_eye * n_eye + blb_ao * n_ao) / ((pe_ms + pa_ms) * 1e-3) / 1e9, 1)}
        ps.close()

    # the headline layout on other trees over the same triangles, same launch shapes
    def compare_tree(label, frame, collapse):
        fs, _ = make_scene(args.layout, frame=frame, collapse=collapse)
        for k in (0, 1):
            fs.set_trace_config(k, **scene.trace_config(k))
        if args.l2_persist:
            fs.set_l2_persist(args.l2_persist)  # as the headline's legs had it
        f_hits = torch.empty_like(d_hits)
        f_any = torch.empty_like(d_any)
        for _ in range(3):
            fs.query_device(0, d_eye.data_ptr(), n_eye, f_hits.data_ptr(), sh)
            fs.query_device(1, d_ao.data_ptr(), n_ao, f_any.data_ptr(), sh)
        torch.cuda.synchronize()
        fe = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
        for k in range(args.steps):
            fe[k][0].record(stream)
            fs.query_device(0, d_eye.data_ptr(), n_eye, f_hits.data_ptr(), sh)
            fe[k][1].record(stream)
            fs.query_device(1, d_ao.data_ptr(), n_ao, f_any.data_ptr(), sh)
            fe[k][2].record(stream)
        torch.cuda.synchronize()
        if args.l2_persist:
            fs.set_l2_persist(0)
        fe_ms = statistics.mean(e[0].elapsed_time(e[1]) for e in fe)
        fa_ms = statistics.mean(e[1].elapsed_time(e[2]) for e in fe)
        fp, ft = fs.query_counters(1, d_ao.data_ptr(), n_ao, sh)
        out = {"tree": label, "eye_ms": round(fe_ms, 4), "ao_ms": round(fa_ms, 4),
               "mrays_s": round((n_eye + n_ao) / (fe_ms + fa_ms) / 1e3, 2),
               "node_fetches_per_ao_ray": round(fp / n_ao, 3), "tri_tests_per_ao_ray": round(ft / n_ao, 3),
               **hit_diff(to_original(d_hits.cpu().numpy().view(np.uint32), prim_idx),
                          to_original(f_hits.cpu().numpy().view(np.uint32), fs.export(0, E.EXPORT_PRIM_INDICES)),
                          "other"),
               "anyhit_mismatch_vs_other": int(np.count_nonzero(f_any.cpu().numpy() != d_any.cpu().numpy()))}
        fs.close()
        del f_hits, f_any
        return out

    tree_cmp = {}
    if not args.no_frame_compare and not args.ncu:
        if args.morton_frame == "cubic" or (args.layout != "bvh2" and args.bvh4_collapse == "largest_first"):
            tree_cmp["reference_tree"] = compare_tree(
                "the reference's tree: per-axis ZIndexMultCoeff grid"
                + (", even-depth BVH2ToBVH4 collapse" if args.layout != "bvh2" else ""), False, False)
        if args.morton_frame == "cubic" and args.layout != "bvh2" and args.bvh4_collapse == "largest_first":
            tree_cmp["even_depth_collapse"] = compare_tree("cubic grid, even-depth collapse", True, False)

    # roofline of the dominant kernel
    eye_avg, ao_avg = statistics.mean(eye_ms), statistics.mean(ao_ms)
    # the headline scene is one untransformed geometry: the single-instance
    # kernels, persistent pool or one thread per ray as the launch shape says
    def kernel_name(kind):
        persistent = scene.trace_config(kind)["persistent"]
        return ("k_trace_one" if persistent else "k_trace_one_grid") + ("<any>" if kind else "<nearest>")

    if ao_avg >= eye_avg:
        dom, dom_ms, dom_bytes, dom_name = "any", ao_avg, ao_bytes, kernel_name(1)
    else:
        dom, dom_ms, dom_bytes, dom_name = "nearest", eye_avg, eye_bytes, kernel_name(0)
    peak, peak_kind = measured_peak()
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    node4_size = {"bvh2": 0, "bvh4": 128, "bvh4_f16": 64, "bvh4_q8": 64}[args.layout]
    n4 = int(scene.export(gid, E.EXPORT_NODES4).nbytes // node4_size) if node4_size else 0
    bb = build_bytes(int(w.idx.size // 3), int(w.verts.shape[0]), int(info["leaves"]), n4, node4_size)
    build_ach = bb / (statistics.median(build_ms) * 1e-3) / 1e9
    build_roofline = {"algorithmic_bytes": bb, "achieved_gb_s": round(build_ach, 1),
                      "frac": round(build_ach / peak, 4), "nodes4": n4,
                      "note": "per-stage reads + writes of the build kernels over the GPU build time; the stages are "
                              "short launches over a few M elements, so the build is latency- and launch-bound"}
    lay = "" if args.layout == "bvh2" else f"_{args.layout}"
    traffic = profile_traffic(f"trace_{dom}{lay}_heightfield2M.txt")
    eye_achieved = eye_bytes / (eye_avg * 1e-3) / 1e9  # the coherent (eye-ray) kernel

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "strong" if split else "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w.name, "tris": int(w.idx.size // 3), "eye_rays": int(n_eye), "ao_rays": int(n_ao),
                   "layout": LAYOUT_DESC[args.layout],
                   "parallelism": f"rays_split{world}" if split else f"replicas{world}",
                   "l2": f"inputs larger than L2: rays {(d_eye.nbytes + d_ao.nbytes) / 1e6:.0f} MB, "
                         f"BVH+triangles {info['bytes'] / 1e6:.0f} MB",
                   "build_ms_median": round(statistics.median(build_ms), 3),
                   "build_roofline": build_roofline,
                   "eye_ms": round(eye_avg, 4), "ao_ms": round(ao_avg, 4),
                   "eye_mrays_s": round(n_eye / eye_avg / 1e3, 2), "ao_mrays_s": round(n_ao / ao_avg / 1e3, 2),
                   "node_pairs_per_eye_ray": round(eye_pairs / n_eye, 3),
                   "node_pairs_per_ao_ray": round(ao_pairs / n_ao, 3)},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": int(RAY_BYTES * (n_eye + n_ao)),
                "api": "hrt_query_nearest_host + hrt_query_any_host, page-locked arrays",
                "async_two_streams_value": round(e2e_async_value, 3),
                "nearest_call_ms": round(1e3 * e2e_eye_s, 4), "any_call_ms": round(1e3 * e2e_ao_s, 4),
                "d2h_bytes_per_step": int(32 * n_eye + n_ao)},
        "e2e_device_raygen": raygen_e2e,
        "gpu_launches": 2 * args.steps,
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1), "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": traffic, "algorithmic_bytes_per_launch": int(dom_bytes),
                     "note": f"algorithmic bytes = {node_bytes} B per node fetch + 36 B per triangle test + ray in/out; "
                             "node fetches mostly hit L1/L2, so frac can exceed 1 (see traffic)",
                     "coherent_eye": {"kernel": kernel_name(0), "achieved": round(eye_achieved, 1),
                                      "frac": round(eye_achieved / peak, 4), "algorithmic_bytes_per_launch": int(eye_bytes),
                                      "traffic": profile_traffic(f"trace_nearest{lay}_heightfield2M.txt")}},
        "clocks": clk,
    }
    line["config"]["bvh4_merge"] = args.merge if args.layout != "bvh2" else None
    line["config"]["l2_persist_mib"] = args.l2_persist
    line["config"]["morton_frame"] = args.morton_frame
    line["config"]["bvh4_collapse"] = args.bvh4_collapse if args.layout != "bvh2" else None
    line["config"]["node_pairs_note"] = "node fetches / triangle tests per ray of the headline's own tree"
    line["config"]["tri_tests_per_ao_ray"] = round(ao_tris / n_ao, 3) if n_ao else None
    for name, cmp in tree_cmp.items():
        line[name] = cmp
        for k in ("mrays_s", "eye_ms", "ao_ms", "node_fetches_per_ao_ray"):
            line["config"][f"{name}_{k}"] = cmp[k]
    line["config"]["eye_ray_order"] = (f"4x8 pixel tiles of the {args.width}-wide image (index arithmetic, results "
                                       "in ray order)" if args.eye_order == "tiles" else "as given (row-major)")
    line["config"]["launch"] = tuned if tuned is not None else "default"
    if split:
        line["split_check"] = split_check
        line["config"]["frame_rays"] = int(frame_rays)
    if plain is not None:
        line["plain"] = plain
        line["speedup_vs_plain"] = round(line["value"] / plain["mrays_s"], 3)

    if not args.no_l2_sweep:
        line["l2_window"] = run_l2_window(scene, d_eye, d_ao, d_hits, d_any, args)
    if not args.no_watertight:
        line["watertight"] = run_watertight(ctx, args, w, ao, d_hits.cpu().numpy().view(np.uint32),
                                            d_any.cpu().numpy().astype(bool),
                                            {k: scene.trace_config(k) for k in (0, 1)})
    if not args.no_frames:
        line["frames"] = run_frames(ctx, args, w, {k: scene.trace_config(k) for k in (0, 1)})
    # the served stream runs before the 256-scene batched measurement: on these
    # boxes its batch times (p99) doubled after that measurement had run, in the
    # same process or a later one, while the headline kernels, the builds and
    # the host link measured the same before and after
    if not args.no_served:
        line["served"] = run_served(ctx, args)
        # the same stream at three times the arrival rate (about 850 Mrays/s
        # offered): requests queue while batches are on the GPU, so batches
        # hold several requests
        line["served_3x"] = run_served(ctx, args, 3 * args.served_rate, 1.5)
    if not args.no_batched:
        line["batched"] = run_batched(ctx, args)
        line["gpu_launches_batched_per_step"] = 2
    if not args.no_precision:
        line["precision"] = run_precision(ctx, args)
    if rank == 0 and not (args.no_cpu_baseline and args.no_oracle_check):
        from oracle import oracle as orc

        o = orc.OracleBVH(w.verts, w.idx)
        if not args.no_cpu_baseline:
            rate, used, sample = cpu_trace_rate(o, w.eye_rays, ao, args.cpu_seconds)
            line["cpu_baseline"] = {"value": round(rate, 3), "unit": UNIT, "cores": int(used), "kind": "port",
                                    "sample": sample, "cpu": host_cpu(), "port_over_reference": PORT_OVER_REFERENCE}
        if not args.no_oracle_check:
            # every ray of the frame against the oracle (after the timed region):
            # the timed layout's device-resident eye hits and AO flags, and the
            # AO flags the e2e leg wrote into host memory
            # primIds compared as original triangle indices (the headline's
            # tree may sort the triangles differently from the reference's)
            want = to_original(o.trace(w.eye_rays).view(np.uint32).reshape(-1, 8), o.prim_indices())
            want_any = o.trace(ao, any_hit=True)
            got = to_original(d_hits.cpu().numpy().view(np.uint32), prim_idx)
            cfg = line["config"]
            cfg["oracle_checked_rays"] = int(n_eye + n_ao)
            dd = hit_diff(got, want, "oracle")
            cfg["oracle_nearest_mismatch"] = dd["nearest_mismatch_vs_oracle"]
            cfg["oracle_nearest_tie"] = dd["nearest_tie_vs_oracle"]
            cfg["oracle_anyhit_mismatch"] = int(np.count_nonzero(d_any.cpu().numpy().astype(bool) != want_any))
            cfg["oracle_e2e_anyhit_mismatch"] = int(np.count_nonzero(got_any.astype(bool) != want_any))
    summarize(line)
    if rank == 0:
        print(json.dumps(line), flush=True)
    replicas.finish(rk)
    return 0


def summarize(line: dict):
    """Scalar copies of the sections' key figures in the line's config (the
    part of the line that record keepers keep whole)."""
    cfg = line["config"]
    if "plain" in line:
        cfg["plain_mrays_s"] = line["plain"]["mrays_s"]
    if "served" in line:
        sv, pl = line["served"]["served"], line["served"]["plain"]
        for k in ("p50_ms", "p99_ms", "max_ms", "mrays_s"):
            cfg[f"served_{k}"] = sv[k]
            cfg[f"served_plain_{k}"] = pl[k]
        cfg["served_mean_requests_per_batch"] = sv["mean_requests_per_batch"]
        cfg["served_engine_p99_ms"] = sv["engine_p99_ms"]
    if "served_3x" in line:
        sv, pl = line["served_3x"]["served"], line["served_3x"]["plain"]
        for k in ("p50_ms", "p99_ms", "mrays_s"):
            cfg[f"served_3x_{k}"] = sv[k]
            cfg[f"served_3x_plain_{k}"] = pl[k]
        cfg["served_3x_mean_requests_per_batch"] = sv["mean_requests_per_batch"]
    if "batched" in line:
        b = line["batched"]
        for k in ("batched_mrays_s", "plain_mrays_s", "speedup", "results_equal_plain"):
            if k in b:
                cfg[f"batched_{k}" if not k.startswith("batched_") else k] = b[k]
    if "precision" in line:
        bad = 0
        for name, sc in line["precision"]["scenes"].items():
            cfg[f"c2_{name}_t_max_rel_vs_fp64"] = sc["t_error_vs_fp64"]["max_rel"]
            for lay, e in sc["layouts"].items():
                cfg[f"c2_{name}_{lay}_mrays_s"] = e["mrays_s"]
                bad += sum(v for k, v in e.items() if "mismatch" in k)
            if "watertight" in sc:
                wt = sc["watertight"]
                cfg[f"c2_{name}_watertight_t_max_rel_vs_fp64"] = wt["t_error_vs_fp64"]["max_rel"]
                cfg[f"c2_{name}_watertight_bvh4_f16_mrays_s"] = wt["layouts"]["bvh4_f16"]["mrays_s"]
                bad += sum(v for e in wt["layouts"].values() for k, v in e.items() if "mismatch" in k)
        cfg["c2_hit_mismatches"] = int(bad)
    if "l2_window" in line:
        for e in line["l2_window"]["sweep"][:-1]:
            cfg[f"l2_window_{e['mib']}mib_ao_ms"] = e["ao_ms"]
            cfg[f"l2_window_{e['mib']}mib_eye_ms"] = e["eye_ms"]
    if "watertight" in line:
        wt = line["watertight"]
        cfg["watertight_mrays_s"] = wt["mrays_s"]
        cfg["watertight_eye_rays_differing_from_mt"] = wt["eye_rays_differing_from_mt"]
        for k, v in wt["differing_by_class"].items():
            cfg[f"watertight_{k}"] = v
        cfg["watertight_ao_rays_differing_from_mt"] = wt["ao_rays_differing_from_mt"]
    if "frames" in line:
        cfg["frames_rtao_mrays_s"] = line["frames"]["rtao"]["mrays_s"]
        cfg["frames_rtao_ms"] = line["frames"]["rtao"]["ms_per_frame"]
        cfg["frames_eye_mrays_s"] = line["frames"]["eye"]["mrays_s"]


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_engine(args)


if __name__ == "__main__":
    sys.exit(main())
