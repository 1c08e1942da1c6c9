"""Python access to the oracle (TEST INFRASTRUCTURE ONLY).

Two checkers of HeavyRT's hot path live here:
  * the C restatement oracle/hrt_oracle.c, built as oracle/_build/liboracle.so
    (every machine);
  * the reference's own CPU code compiled by oracle/Makefile.ref into
    oracle/_ref/ (only where the reference sources are present).
Only tests, the smoke check and the benchmark's CPU-baseline leg use this
module; the engine never imports it.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
NODE_DTYPE = np.dtype([("boxMin", "<f4", (3,)), ("leftOffset", "<u4"), ("boxMax", "<f4", (3,)), ("escapeIndex", "<u4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("primId", "<u4"), ("instId", "<u4"), ("geomId", "<u4"), ("coords", "<f4", (4,))])

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        p = HERE / "_build" / "liboracle.so"
        if not p.exists():
            raise RuntimeError(f"oracle not built ({p} missing): run __graft_entry__.build()")
        L = C.CDLL(str(p))
        vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
        L.ora_build.restype = vp
        L.ora_build.argtypes = [vp, u32, vp, u32]
        L.ora_build_frame.restype = vp
        L.ora_build_frame.argtypes = [vp, u32, vp, u32, i32]
        L.ora_free.argtypes = [vp]
        for f in ("ora_num_tris", "ora_num_leaves", "ora_num_nodes"):
            getattr(L, f).restype = u32
            getattr(L, f).argtypes = [vp]
        L.ora_status.restype = i32
        L.ora_status.argtypes = [vp]
        L.ora_get_box.argtypes = [vp, vp]
        L.ora_copy_u32.argtypes = [vp, i32, vp]
        L.ora_trace.restype = i32
        L.ora_trace.argtypes = [vp, vp, u64, i32, vp, vp, i32, vp]
        L.ora_set_triangle_test.argtypes = [vp, i32]
        L.ora_eye_rays.argtypes = [vp, vp, u32, u32, C.c_float, C.c_float, vp]
        f32 = C.c_float
        L.ora_pack_xy.argtypes = [u32, u32, vp]
        L.ora_eye_colors.argtypes = [vp, u64, vp]
        L.ora_qmc_table.argtypes = [vp]
        L.ora_rtao_tile.argtypes = [u32, vp]
        L.ora_rtao_positions.argtypes = [vp, vp, u64, vp, vp, vp, vp, vp]
        L.ora_rtao_ao_rays.argtypes = [vp, u32, u32, u32, vp, f32, vp]
        L.ora_rtao_colors.argtypes = [vp, vp, u64, u32, f32, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


class OracleBVH:
    """LBVH built by the C restatement: stage arrays + peach layout + traversal."""

    def __init__(self, verts: np.ndarray, idx: np.ndarray, cubic: bool = False):
        """cubic=True builds on the engine's cubic Morton grid instead of the
        reference's per-axis one."""
        self._v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 4)
        self._i = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1)
        self._h = C.c_void_p(lib().ora_build_frame(_p(self._v), self._v.shape[0], _p(self._i), self._i.size,
                                                   1 if cubic else 0))
        self.n_tris = lib().ora_num_tris(self._h)
        self.n_leaves = lib().ora_num_leaves(self._h)
        self.n_nodes = lib().ora_num_nodes(self._h)
        self.status = lib().ora_status(self._h)

    def _u32(self, which: int, count: int) -> np.ndarray:
        out = np.empty(count, dtype=np.uint32)
        if count:
            lib().ora_copy_u32(self._h, which, _p(out))
        return out

    def scene_box(self) -> np.ndarray:
        out = np.empty(12, dtype=np.float32)
        lib().ora_get_box(self._h, _p(out))
        return out

    def morton_unsorted(self):
        return self._u32(0, 2 * self.n_tris).reshape(-1, 2)

    def morton_sorted(self):
        return self._u32(1, 2 * self.n_tris).reshape(-1, 2)

    def compressed(self):
        return self._u32(2, self.n_leaves)

    def run_starts(self):
        return self._u32(3, self.n_leaves)

    def lr_nodes(self):
        n = 2 * self.n_leaves - 1 if self.n_leaves else 0
        return self._u32(4, 8 * n).view(NODE_DTYPE)

    def lr_counts(self):
        return self._u32(5, 2 * self.n_leaves - 1 if self.n_leaves else 0)

    def prim_indices(self):
        return self._u32(6, self.n_tris)

    def peach_nodes(self):
        return self._u32(7, 8 * self.n_nodes).view(NODE_DTYPE)

    def sorted_indices(self):
        return self._u32(8, 3 * self.n_tris)

    def trace(self, rays: np.ndarray, any_hit: bool = False, threads: int = 0, counters: bool = False,
              watertight: bool = False):
        """BVH2TraverseC32 over the rays; with watertight=True the leaves use
        the watertight triangle test instead of the reference's MT test."""
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = r.shape[0]
        cnt = np.zeros(2, dtype=np.uint64)
        lib().ora_set_triangle_test(self._h, 1 if watertight else 0)
        if any_hit:
            out = np.empty(n, dtype=np.uint8)
            used = lib().ora_trace(self._h, _p(r), n, 1, None, _p(out), threads, _p(cnt) if counters else None)
            res = out.astype(bool)
        else:
            out = np.empty(n, dtype=HIT_DTYPE)
            used = lib().ora_trace(self._h, _p(r), n, 0, _p(out), None, threads, _p(cnt) if counters else None)
            res = out
        if counters:
            return res, (int(cnt[0]), int(cnt[1])), used
        return res

    def close(self):
        if self._h:
            lib().ora_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- 4-wide collapse

LEAF_BIT, EMPTY_REF = 0x80000000, 0xFFFFFFFF
COLLAPSE_EVEN_DEPTH, COLLAPSE_LARGEST_FIRST = 0, 1


def collapse4(lr: np.ndarray, counts: np.ndarray, run_starts: np.ndarray, n_tris: int, merge: int = 0,
              rule: int = COLLAPSE_EVEN_DEPTH) -> np.ndarray:
    """The 4-wide nodes of a binary LBVH (lr_nodes / lr_counts / run_starts of
    this module's OracleBVH) as uint32 [n, 32] FP32 node records: lo x, y, z,
    hi x, y, z (four floats each, one per slot), the four slot refs, padding.

    rule COLLAPSE_EVEN_DEPTH is BVH2ToBVH4 (core/builders/cbvh.cpp:226-311): a
    4-wide node's slots are its binary node's grandchildren (a leaf child
    stands for itself), so the 4-wide nodes are the internal nodes at even
    depth.  COLLAPSE_LARGEST_FIRST starts from the two children and twice
    opens the internal slot with the largest descendant count (the leftmost
    of equals).  merge 0: an internal slot whose two children are leaves
    becomes one leaf; M > 0: a slot over at most M triangles does (1 never).
    A leaf slot refers to its first sorted triangle (LEAF_BIT set), an internal
    slot to the 4-wide node it becomes, numbered in binary-node order; unused
    slots are EMPTY_REF with zero boxes.  Pure Python: small trees only."""
    L = len(run_starts)
    left = lr["leftOffset"].astype(np.int64)
    right = lr["escapeIndex"].astype(np.int64)
    bmin, bmax = lr["boxMin"], lr["boxMax"]

    def is_leaf(n):
        return n >= L - 1

    def tri_range(n):
        a = b = n
        while not is_leaf(a):
            a = left[a]
        while not is_leaf(b):
            b = right[b]
        la, lb = a - (L - 1), b - (L - 1)
        return int(run_starts[la]), int(run_starts[lb + 1]) if lb + 1 < L else n_tris

    def merges(n):
        if n == 0:
            return False
        if merge == 0:
            return is_leaf(left[n]) and is_leaf(right[n])
        if merge == 1:
            return False
        st, en = tri_range(n)
        return en - st <= merge

    def slots(n):
        if rule == COLLAPSE_EVEN_DEPTH:
            out = []
            for c in (left[n], right[n]):
                out += [c] if is_leaf(c) else [left[c], right[c]]
            return out
        out = [left[n], right[n]]
        for _ in range(2):
            best = None
            for k, c in enumerate(out):
                if not is_leaf(c) and (best is None or counts[c] > counts[out[best]]):
                    best = k
            if best is None:
                break
            c = out[best]
            out[best:best + 1] = [left[c], right[c]]
        return out

    def record(sl, index, role):
        w = np.zeros(32, np.uint32)
        box = np.zeros((6, 4), np.float32)
        refs = [EMPTY_REF] * 4
        for k, c in enumerate(sl):
            box[0:3, k] = bmin[c]
            box[3:6, k] = bmax[c]
            if is_leaf(c):
                refs[k] = LEAF_BIT | int(run_starts[c - (L - 1)])
            elif role[c] == 2:
                refs[k] = LEAF_BIT | tri_range(c)[0]
            else:
                refs[k] = int(index[c])
        w[0:24] = box.reshape(-1).view(np.uint32)
        w[24:28] = refs
        return w

    if L == 1:
        w = np.zeros(32, np.uint32)
        box = np.zeros((6, 4), np.float32)
        box[0:3, 0], box[3:6, 0] = bmin[0], bmax[0]
        w[0:24] = box.reshape(-1).view(np.uint32)
        w[24:28] = [LEAF_BIT | int(run_starts[0]), EMPTY_REF, EMPTY_REF, EMPTY_REF]
        return w.reshape(1, 32)
    role = np.zeros(L - 1, np.uint8)
    if rule == COLLAPSE_EVEN_DEPTH:
        depth = np.zeros(L - 1, np.int64)
        stack = [(0, 0)]  # internal nodes are not stored parent first: walk down from the root
        while stack:
            n, d = stack.pop()
            depth[n] = d
            for c in (left[n], right[n]):
                if not is_leaf(c):
                    stack.append((c, d + 1))
        for n in range(L - 1):
            if depth[n] % 2 == 0:
                role[n] = 2 if merges(n) else 1
    else:
        role[0] = 1
        frontier = [0]
        while frontier:
            nxt = []
            for b in frontier:
                for c in slots(b):
                    if not is_leaf(c):
                        role[c] = 2 if merges(c) else 1
                        if role[c] == 1:
                            nxt.append(c)
            frontier = nxt
    index = np.cumsum(role == 1) - (role == 1)
    return np.stack([record(slots(n), index, role) for n in range(L - 1) if role[n] == 1])


# ---------------------------------------------------------------- reference checker

def eye_rays(proj_inv: np.ndarray, world_view_inv: np.ndarray, width: int, height: int, t_near: float = 0.0,
             t_far: float = 3.4028234663852886e38) -> np.ndarray:
    """The renderers' eye rays (C restatement); matrices as 4x4 row-major numpy arrays."""
    pi = np.ascontiguousarray(np.asarray(proj_inv, np.float32).T)  # column-major storage
    wi = np.ascontiguousarray(np.asarray(world_view_inv, np.float32).T)
    out = np.empty((width * height, 8), np.float32)
    lib().ora_eye_rays(_p(pi), _p(wi), width, height, t_near, t_far, _p(out))
    return out


def reference_eye_rays(proj_inv, world_view_inv, width: int, height: int, t_near: float = 0.0,
                       t_far: float = 3.4028234663852886e38):
    """The same rays from the reference's own helpers (oracle/_ref/raygen_harness), or None."""
    exe = HERE / "_ref" / "raygen_harness"
    if not exe.exists():
        return None
    pi = np.asarray(proj_inv, np.float32).T.reshape(-1)
    wi = np.asarray(world_view_inv, np.float32).T.reshape(-1)
    with tempfile.TemporaryDirectory() as d:
        src, dst = Path(d) / "p.bin", Path(d) / "o.bin"
        src.write_bytes(np.concatenate([pi, wi]).astype(np.float32).tobytes() +
                        np.array([width, height], np.uint32).tobytes() + np.array([t_near, t_far], np.float32).tobytes())
        subprocess.run([str(exe), "eye", str(src), str(dst)], check=True)
        return np.fromfile(dst, dtype=np.float32).reshape(-1, 8)


def reference_harness(fast: bool = False) -> Path | None:
    p = HERE / "_ref" / ("ref_harness_fast" if fast else "ref_harness")
    return p if p.exists() else None


def _write_scene(path, verts, idx):
    v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 4)
    i = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1)
    with open(path, "wb") as f:
        f.write(b"HRTSCN01")
        f.write(np.array([v.shape[0], i.size], dtype=np.uint64).tobytes())
        f.write(v.tobytes())
        f.write(i.tobytes())


def _write_rays(path, rays):
    r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    with open(path, "wb") as f:
        f.write(b"HRTRAY01")
        f.write(np.array([r.shape[0]], dtype=np.uint64).tobytes())
        f.write(r.tobytes())


def run_reference(verts, idx, rays=None, fast: bool = False, threads: int = 0) -> dict:
    """Run the reference's own builder (and traversal, if rays are given).

    Returns the stage arrays (scene box, codes, compressed codes, run starts, LR
    tree, counts), the BVH2CommonRT arrays (peach nodes, prim indices, sorted
    indices) and, with rays, the hits / any-hit flags and its counters."""
    exe = reference_harness(fast)
    if exe is None:
        raise RuntimeError("reference checker not built (reference sources absent)")
    out = {}
    with tempfile.TemporaryDirectory() as td:
        sp = os.path.join(td, "scene.bin")
        _write_scene(sp, verts, idx)
        pre = os.path.join(td, "out")
        r = subprocess.run([str(exe), "stages", sp, pre], capture_output=True, text=True, check=True)
        out["stages_info"] = json.loads(r.stdout.strip().splitlines()[-1])
        rd = lambda s, dt: np.fromfile(pre + s, dtype=dt)  # noqa: E731
        out["scene_box"] = rd(".bbox", np.float32)
        out["morton_unsorted"] = rd(".codes_unsorted", np.uint32).reshape(-1, 2)
        out["morton_sorted"] = rd(".codes_sorted", np.uint32).reshape(-1, 2)
        out["compressed"] = rd(".compressed", np.uint32)
        out["run_starts"] = rd(".runstarts", np.uint32)
        out["lr_nodes"] = rd(".lr_nodes", NODE_DTYPE)
        out["lr_counts"] = rd(".lr_count", np.uint32)
        out["leaf_indices"] = rd(".leaf_indices", np.uint32)
        r = subprocess.run([str(exe), "build", sp, pre], capture_output=True, text=True, check=True)
        out["build_info"] = json.loads(r.stdout.strip().splitlines()[-1])
        out["peach_nodes"] = rd(".peach_nodes", NODE_DTYPE)
        out["prim_indices"] = rd(".prim_indices", np.uint32)
        out["sorted_indices"] = rd(".indices_sorted", np.uint32)
        if rays is not None:
            rp = os.path.join(td, "rays.bin")
            _write_rays(rp, rays)
            cmd = [str(exe), "trace", sp, pre, rp]
            if fast and threads:
                cmd.append(str(threads))
            r = subprocess.run(cmd, capture_output=True, text=True, check=True)
            out["trace_info"] = json.loads(r.stdout.strip().splitlines()[-1])
            out["hits"] = rd(".hits", HIT_DTYPE)
            out["any"] = rd(".any", np.uint8).astype(bool)
    return out


# ---------------------------------------------------------------- renderer frames
AO_TILE = 128
AO_HIT_BACK = 10000000.0


def pack_xy(width: int, height: int) -> np.ndarray:
    """EyeRayCaster's packed pixel order: entry k = y << 16 | x of the k-th traced pixel."""
    out = np.zeros(width * height, np.uint32)
    lib().ora_pack_xy(width, height, _p(out))
    return out


def eye_colors(hits: np.ndarray) -> np.ndarray:
    h = np.ascontiguousarray(hits).view(HIT_DTYPE)
    out = np.empty(h.shape[0], np.uint32)
    lib().ora_eye_colors(_p(h), h.shape[0], _p(out))
    return out


def qmc_table() -> np.ndarray:
    out = np.empty((4, 31), np.uint32)
    lib().ora_qmc_table(_p(out))
    return out


def rtao_tile(rays_per_pixel: int) -> np.ndarray:
    out = np.empty((AO_TILE * AO_TILE * rays_per_pixel, 2), np.float32)
    lib().ora_rtao_tile(rays_per_pixel, _p(out))
    return out


def rtao_positions(eye_rays, hits, geoms, norm_matrices) -> np.ndarray:
    """kernel_TraceEyeRay2's shading.  geoms: per geometry (sorted index buffer,
    float4 vertices, float4 normals); norm_matrices: (nInst, 4, 4) row-major."""
    r = np.ascontiguousarray(eye_rays, np.float32).reshape(-1, 8)
    h = np.ascontiguousarray(hits).view(HIT_DTYPE)
    keep = []
    arrs = []
    for g in geoms:
        si = np.ascontiguousarray(g[0], np.uint32).reshape(-1)
        v = np.ascontiguousarray(g[1], np.float32).reshape(-1, 4)
        nn = np.ascontiguousarray(g[2], np.float32).reshape(-1, 4)
        keep += [si, v, nn]
        arrs.append((si.ctypes.data, v.ctypes.data, nn.ctypes.data))
    n_g = max(len(arrs), 1)
    ptr_i = (C.c_void_p * n_g)(*[a[0] for a in arrs])
    ptr_v = (C.c_void_p * n_g)(*[a[1] for a in arrs])
    ptr_n = (C.c_void_p * n_g)(*[a[2] for a in arrs])
    m = np.ascontiguousarray(np.transpose(np.asarray(norm_matrices, np.float32).reshape(-1, 4, 4), (0, 2, 1)))
    out = np.empty((r.shape[0], 4), np.float32)
    lib().ora_rtao_positions(_p(r), _p(h), r.shape[0], C.cast(ptr_i, C.c_void_p), C.cast(ptr_v, C.c_void_p),
                             C.cast(ptr_n, C.c_void_p), _p(m), _p(out))
    return out


def rtao_ao_rays(positions, width: int, height: int, rays_per_pixel: int, tile, ao_max_radius: float):
    """kernel_InitAORay for every (pixel, sample): (W*H*R, 8) rays, zero where the pixel has no hit."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
    t = np.ascontiguousarray(tile, np.float32).reshape(-1, 2)
    out = np.zeros((width * height * rays_per_pixel, 8), np.float32)
    lib().ora_rtao_ao_rays(_p(pos), width, height, rays_per_pixel, _p(t), ao_max_radius, _p(out))
    return out


def rtao_colors(positions, ao_hit, rays_per_pixel: int, power: float = 1.0):
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
    a = np.ascontiguousarray(ao_hit, np.uint8).reshape(-1)
    vis = np.empty(pos.shape[0], np.float32)
    col = np.empty(pos.shape[0], np.uint32)
    lib().ora_rtao_colors(_p(pos), _p(a), pos.shape[0], rays_per_pixel, power, _p(vis), _p(col))
    return vis, col


def eye_frame(bvh: "OracleBVH", proj_inv, world_view_inv, width: int, height: int) -> np.ndarray:
    """EyeRayCaster's frame over one geometry (identity instance): colours, row-major."""
    rays = eye_rays(proj_inv, world_view_inv, width, height, 0.0, 3.4028234663852886e38)
    return eye_colors(bvh.trace(rays))


def rtao_frame(bvh: "OracleBVH", verts, normals, proj_inv, world_view_inv, width: int, height: int, z_near: float,
               z_far: float, rays_per_pixel: int, ao_max_radius: float, power: float = 1.0, norm_matrix=None) -> dict:
    """RTAO's frame over one geometry (identity instance), every stage."""
    nm = np.eye(4, dtype=np.float32) if norm_matrix is None else np.asarray(norm_matrix, np.float32)
    rays = eye_rays(proj_inv, world_view_inv, width, height, z_near, z_far)
    hits = bvh.trace(rays)
    pos = rtao_positions(rays, hits, [(bvh.sorted_indices(), verts, normals)], nm[None])
    tile = rtao_tile(rays_per_pixel)
    ao = rtao_ao_rays(pos, width, height, rays_per_pixel, tile, ao_max_radius)
    valid = np.repeat(pos[:, 1] < AO_HIT_BACK, rays_per_pixel)
    ao_hit = np.zeros(ao.shape[0], np.uint8)
    if valid.any():
        ao_hit[valid] = bvh.trace(ao[valid], any_hit=True).astype(np.uint8)
    vis, col = rtao_colors(pos, ao_hit, rays_per_pixel, power)
    return {"eye_rays": rays, "eye_hits": hits, "positions": pos, "tile": tile, "ao_rays": ao, "ao_valid": valid,
            "ao_hit": ao_hit, "visibility": vis, "colors": col}


def _render_params(proj_inv, world_view_inv, width, height, z_near, z_far, rays_per_pixel, radius, power,
                   norm_matrix) -> bytes:
    pi = np.asarray(proj_inv, np.float32).T.reshape(-1)
    wi = np.asarray(world_view_inv, np.float32).T.reshape(-1)
    nm = np.asarray(np.eye(4) if norm_matrix is None else norm_matrix, np.float32).T.reshape(-1)
    return (np.concatenate([pi, wi]).astype(np.float32).tobytes() + np.array([width, height], np.uint32).tobytes() +
            np.array([z_near, z_far], np.float32).tobytes() + np.array([rays_per_pixel], np.uint32).tobytes() +
            np.array([radius, power], np.float32).tobytes() + nm.tobytes())


def reference_render(kind: str, verts, idx, proj_inv, world_view_inv, width: int, height: int, normals=None,
                     z_near: float = 0.0, z_far: float = 3.4028234663852886e38, rays_per_pixel: int = 4,
                     radius: float = 1.0, power: float = 1.0, norm_matrix=None):
    """The reference renderers' own frame kernels (oracle/_ref/render_harness), or None
    where the reference sources are absent.  kind: "eye", "rtao" or "qmc"."""
    exe = HERE / "_ref" / "render_harness"
    if not exe.exists():
        return None
    with tempfile.TemporaryDirectory() as td:
        pre = os.path.join(td, "out")
        rd = lambda s, dt: np.fromfile(pre + s, dtype=dt)  # noqa: E731
        if kind == "qmc":
            subprocess.run([str(exe), "qmc", str(rays_per_pixel), pre], check=True)
            return {"qmc": rd(".qmc", np.uint32).reshape(4, 31), "tile": rd(".tile", np.float32).reshape(-1, 2)}
        sp, pp = os.path.join(td, "scene.bin"), os.path.join(td, "params.bin")
        _write_scene(sp, verts, idx)
        with open(pp, "wb") as f:
            f.write(_render_params(proj_inv, world_view_inv, width, height, z_near, z_far, rays_per_pixel, radius,
                                   power, norm_matrix))
        if kind == "eye":
            subprocess.run([str(exe), "eye", sp, pp, pre], check=True)
            return {"packed": rd(".packed", np.uint32), "colors": rd(".colors", np.uint32)}
        npth = os.path.join(td, "normals.bin")
        nn = np.ascontiguousarray(normals, np.float32).reshape(-1, 4)
        with open(npth, "wb") as f:
            f.write(b"HRTNRM01" + np.array([nn.shape[0]], np.uint64).tobytes() + nn.tobytes())
        subprocess.run([str(exe), "rtao", sp, npth, pp, pre], check=True)
        return {"eye_rays": rd(".eye_rays", np.float32).reshape(-1, 8), "eye_hits": rd(".eye_hits", HIT_DTYPE),
                "positions": rd(".positions", np.float32).reshape(-1, 4),
                "ao_rays": rd(".ao_rays", np.float32).reshape(-1, 8), "ao_hit": rd(".ao_hit", np.uint8),
                "visibility": rd(".visibility", np.float32), "colors": rd(".colors", np.uint32)}
