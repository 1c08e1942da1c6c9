"""Autotuner for batched scenes: node width, leaf size, collapse rule and
launch shape.

The launch shape (threads per block, persistent pool, refill policy) is tuned
by the engine itself (hrt_scene_autotune) for a fixed tree.  The tree shape is
chosen here, because changing it means rebuilding: every candidate structure
(BVH2, or BVH4 in FP32 / FP16 / 8-bit nodes with leaves of at most 1..8
triangles, by the reference's even-depth collapse or the largest-first one) is
built from the same geometry with the segmented build, its launch shape tuned
per query kind, and the structure with the lowest summed query time kept.  All
candidates share the binary tree and its triangle order; the binary layout
makes the reference's decisions and the 4-wide ones may pick another triangle
only at a tie within 1e-5 relative t, so the choice changes speed, not
answers.

The launch shape includes the short stack's size: the entries a ray keeps in
shared memory (16..64; deeper entries spill to local memory, so every size is
correct for every tree), tuned by the engine after the block shape.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import engine as E

# (layout name, BVH4 merge bound, collapse rule): merge M collapses subtrees of <= M
# triangles into one leaf; the rule is E.BVH4_COLLAPSE_EVEN_DEPTH (the reference's)
# or E.BVH4_COLLAPSE_LARGEST_FIRST
EVEN, LARGEST = E.BVH4_COLLAPSE_EVEN_DEPTH, E.BVH4_COLLAPSE_LARGEST_FIRST
DEFAULT_STRUCTURES = ([("bvh2", None, EVEN)] + [(lay, m, EVEN) for lay in ("bvh4_f16", "bvh4_q8", "bvh4")
                                                for m in (1, 2, 4, 8)]
                      + [("bvh4_f16", m, LARGEST) for m in (1, 2, 4)])


@dataclass
class TuneResult:
    layout: str
    merge: int | None
    configs: dict                       # kind -> launch config
    ms: dict                            # kind -> mean ms of one query
    # every candidate: (layout, merge, collapse rule, ms nearest, ms any, stack entries nearest, stack entries any)
    table: list = field(default_factory=list)
    collapse: int = EVEN


def build_batch(ctx, verts, idx, layout: str, merge, collapse: int = EVEN):
    scene = E.SceneRT(ctx, layout=layout)
    if merge is not None and layout != "bvh2":
        scene.set_bvh4_merge(merge)
        scene.set_bvh4_collapse(collapse)
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
    for layout, merge, collapse in structures:
        scene, _ = build_batch(ctx, verts, idx, layout, merge, collapse)
        cfgs, ms = {}, {}
        for kind, out in ((0, d_hits), (1, d_any)):
            desc = E.query_desc(kind, d_rays, n_rays, out, d_offsets, d_seg_inst, n_seg)
            cfgs[kind], ms[kind] = scene.autotune(desc, repeats)
        table.append((layout, merge, "largest_first" if collapse == LARGEST else "even_depth", round(ms[0], 4),
                      round(ms[1], 4), cfgs[0]["stackEntries"], cfgs[1]["stackEntries"]))
        if best is None or ms[0] + ms[1] < best.ms[0] + best.ms[1]:
            best = TuneResult(layout, merge, cfgs, ms, collapse=collapse)
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
