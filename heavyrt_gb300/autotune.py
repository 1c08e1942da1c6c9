"""Autotuner for batched scenes: node width, leaf size and launch shape.

The launch shape (threads per block, persistent pool, refill policy) is tuned
by the engine itself (hrt_scene_autotune) for a fixed tree.  The tree shape is
chosen here, because changing it means rebuilding: every candidate structure
(BVH2, or BVH4 in FP32 / FP16 / 8-bit nodes with leaves of at most 1..8
triangles) is built from the same geometry with the segmented build, its
launch shape tuned per query kind, and the structure with the lowest summed
query time kept.  Results never depend on the choice (the traversal makes the
reference's decisions in every layout); only speed does.

The launch shape includes the short stack's size: the entries a ray keeps in
shared memory (16..64; deeper entries spill to local memory, so every size is
correct for every tree), tuned by the engine after the block shape.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import engine as E

# (layout name, BVH4 merge bound): merge M collapses subtrees of <= M triangles into one leaf
DEFAULT_STRUCTURES = [("bvh2", None)] + [(lay, m) for lay in ("bvh4_f16", "bvh4_q8", "bvh4")
                                         for m in (1, 2, 4, 8)]


@dataclass
class TuneResult:
    layout: str
    merge: int | None
    configs: dict                       # kind -> launch config
    ms: dict                            # kind -> mean ms of one query
    # every candidate: (layout, merge, ms nearest, ms any, stack entries nearest, stack entries any)
    table: list = field(default_factory=list)


def build_batch(ctx, verts, idx, layout: str, merge):
    scene = E.SceneRT(ctx, layout=layout)
    if merge is not None and layout != "bvh2":
        scene.set_bvh4_merge(merge)
    ids = scene.add_geoms_batched(verts, idx)
    for g in ids:
        scene.AddInstance(g)
    scene.CommitScene()
    return scene, ids


def tune_batch(ctx, verts, idx, d_rays, n_rays: int, d_offsets, d_seg_inst, n_seg: int, d_hits, d_any,
               structures=DEFAULT_STRUCTURES, repeats: int = 2) -> TuneResult:
    """Chooses the structure and launch shapes for segmented queries over the
    batch (device pointers as ints).  Returns the choice and the full table."""
    best = None
    table = []
    for layout, merge in structures:
        scene, _ = build_batch(ctx, verts, idx, layout, merge)
        cfgs, ms = {}, {}
        for kind, out in ((0, d_hits), (1, d_any)):
            desc = E.query_desc(kind, d_rays, n_rays, out, d_offsets, d_seg_inst, n_seg)
            cfgs[kind], ms[kind] = scene.autotune(desc, repeats)
        table.append((layout, merge, round(ms[0], 4), round(ms[1], 4), cfgs[0]["stackEntries"],
                      cfgs[1]["stackEntries"]))
        if best is None or ms[0] + ms[1] < best.ms[0] + best.ms[1]:
            best = TuneResult(layout, merge, cfgs, ms)
        scene.close()
    best.table = table
    return best


def apply(scene: E.SceneRT, result: TuneResult):
    """Sets a tuned launch shape on a scene built with result's structure."""
    for kind, c in result.configs.items():
        scene.set_trace_config(kind, c["threadsPerBlock"], c["persistent"], c["stepsPerRefill"], c["refillLanes"],
                               c["stackEntries"], c["imageWidth"])


def seg_inst_identity(n: int) -> np.ndarray:
    return np.arange(n, dtype=np.uint32)
