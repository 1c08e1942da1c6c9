"""Python binding of the engine's C ABI (include/hrt.h) and a mirror of
HeavyRT's ISceneObject plugin interface (core/CrossRT.h:64-196).

The binding loads heavyrt_gb300/_build/libhrt.so and fails loudly when it is
missing: there is no CPU fallback.  Method names, argument meaning and
defaults follow ISceneObject so that code written against HeavyRT's interface
reads the same here; the ray queries are batched (arrays of rays) because a
per-ray call cannot be fast on a GPU.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_BUILD = Path(__file__).resolve().parent / "_build"

# statuses (include/hrt.h)
HRT_OK = 0
HRT_ERR_INVALID_ARGUMENT = 1
HRT_ERR_CUDA = 2
HRT_ERR_OUT_OF_MEMORY = 3
HRT_ERR_CAPACITY = 4
HRT_ERR_STATE = 5
HRT_ERR_TIMEOUT = 6
HRT_ERR_DEVICE_CHECK = 7
HRT_ERR_UNSUPPORTED = 8

# BuildQuality, core/CrossRT.h:9-15
BUILD_LOW, BUILD_MEDIUM, BUILD_HIGH, BUILD_REFIT = 0, 1, 2, 3

# exports (include/hrt.h)
EXPORT_SCENE_BOX = 0
EXPORT_MORTON_SORTED = 1
EXPORT_COMPRESSED = 2
EXPORT_RUN_STARTS = 3
EXPORT_LR_NODES = 4
EXPORT_LR_COUNTS = 5
EXPORT_PRIM_INDICES = 6
EXPORT_SORTED_INDICES = 7
EXPORT_MORTON_UNSORTED = 8
EXPORT_NODES4 = 9
EXPORT_PAIR_RECORDS = 10

# node layouts (include/hrt.h); names accepted as CreateSceneRT's a_layoutName
LAYOUT_BVH2, LAYOUT_BVH4_F32, LAYOUT_BVH4_F16, LAYOUT_BVH4_Q8 = 0, 1, 2, 3
OPTION_BVH4_MERGE, OPTION_TLAS, OPTION_TRIANGLE_TEST, OPTION_L2_PERSIST, OPTION_MORTON_FRAME = 1, 2, 3, 4, 5
OPTION_BVH4_COLLAPSE = 6
MORTON_PER_AXIS, MORTON_CUBIC = 0, 1
BVH4_COLLAPSE_EVEN_DEPTH, BVH4_COLLAPSE_LARGEST_FIRST = 0, 1
TRI_MOLLER_TRUMBORE, TRI_WATERTIGHT = 0, 1
TRI_TEST_NAMES = {"mt": TRI_MOLLER_TRUMBORE, "moller_trumbore": TRI_MOLLER_TRUMBORE, "watertight": TRI_WATERTIGHT}
LAYOUT_NAMES = {"": LAYOUT_BVH2, "bvh2": LAYOUT_BVH2, "bvh4": LAYOUT_BVH4_F32, "bvh4_f32": LAYOUT_BVH4_F32,
                "bvh4_f16": LAYOUT_BVH4_F16, "bvh4_half": LAYOUT_BVH4_F16, "bvh4_q8": LAYOUT_BVH4_Q8}

# CRT_Hit, core/CrossRT.h:20-27
HIT_DTYPE = np.dtype([("t", "<f4"), ("primId", "<u4"), ("instId", "<u4"), ("geomId", "<u4"), ("coords", "<f4", (4,))])
# BVHNode, core/builders/cbvh.h:20-26
NODE_DTYPE = np.dtype([("boxMin", "<f4", (3,)), ("leftOffset", "<u4"), ("boxMax", "<f4", (3,)), ("escapeIndex", "<u4")])

_EXPORT_DTYPES = {
    EXPORT_SCENE_BOX: np.float32,
    EXPORT_MORTON_SORTED: np.uint32,
    EXPORT_MORTON_UNSORTED: np.uint32,
    EXPORT_COMPRESSED: np.uint32,
    EXPORT_RUN_STARTS: np.uint32,
    EXPORT_LR_NODES: NODE_DTYPE,
    EXPORT_LR_COUNTS: np.uint32,
    EXPORT_PRIM_INDICES: np.uint32,
    EXPORT_SORTED_INDICES: np.uint32,
    EXPORT_NODES4: np.uint32,
    EXPORT_PAIR_RECORDS: np.uint32,
}


class TraceConfig(C.Structure):
    """hrt_trace_config (include/hrt.h): launch shape of the traversal kernel."""

    _fields_ = [("threadsPerBlock", C.c_int), ("persistent", C.c_int), ("stepsPerRefill", C.c_int),
                ("refillLanes", C.c_int), ("stackEntries", C.c_int), ("imageWidth", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class QueryDesc(C.Structure):
    """hrt_query_desc (include/hrt.h): one traversal launch, optionally segmented."""

    _fields_ = [("kind", C.c_int), ("rays", C.c_void_p), ("n", C.c_uint64), ("rayOffsets", C.c_void_p),
                ("segInst", C.c_void_p), ("nSeg", C.c_uint32), ("out", C.c_void_p)]


def query_desc(kind: int, rays_ptr: int, n: int, out_ptr: int, ray_offsets_ptr: int = 0, seg_inst_ptr: int = 0,
               n_seg: int = 0) -> QueryDesc:
    return QueryDesc(int(kind), C.c_void_p(rays_ptr), int(n), C.c_void_p(ray_offsets_ptr or None),
                     C.c_void_p(seg_inst_ptr or None), int(n_seg), C.c_void_p(out_ptr))


class ServerConfig(C.Structure):
    """hrt_server_config (include/hrt.h)."""

    _fields_ = [("memoryBudget", C.c_uint64), ("slotRays", C.c_uint64), ("slots", C.c_uint32),
                ("maxScenes", C.c_uint32), ("maxBatchRequests", C.c_uint32), ("layout", C.c_int),
                ("bvh4Merge", C.c_int), ("mortonFrame", C.c_int), ("bvh4Collapse", C.c_int)]


class RequestInfo(C.Structure):
    """hrt_request_info (include/hrt.h)."""

    _fields_ = [("status", C.c_int), ("batch", C.c_uint32), ("batchRequests", C.c_uint32), ("batchRays", C.c_uint64),
                ("tSubmit", C.c_double), ("tStart", C.c_double), ("tDone", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerStats(C.Structure):
    """hrt_server_stats (include/hrt.h)."""

    _fields_ = [("requests", C.c_uint64), ("rays", C.c_uint64), ("batches", C.c_uint64), ("builds", C.c_uint64),
                ("evictions", C.c_uint64), ("failed", C.c_uint64), ("residentBytes", C.c_uint64),
                ("peakResidentBytes", C.c_uint64), ("scenesResident", C.c_uint32), ("queued", C.c_uint32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


SCENE_BUILDING, SCENE_READY, SCENE_FAILED, SCENE_EVICTED = 0, 1, 2, 3


class RtaoParams(C.Structure):  # hrt_rtao_params
    _fields_ = [("projInv", C.c_float * 16), ("worldViewInv", C.c_float * 16), ("zNear", C.c_float),
                ("zFar", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32), ("aoMaxRadius", C.c_float),
                ("power", C.c_float)]


class HrtError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"hrt status {status}: {message}")
        self.status = status


_lib = None


def library_path() -> Path:
    return _BUILD / "libhrt.so"


def lib() -> C.CDLL:
    """The loaded engine library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = library_path()
    if not p.exists():
        raise RuntimeError(f"native engine not built ({p} missing): run __graft_entry__.build()")
    L = C.CDLL(str(p))
    vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
    sig = {
        "hrt_context_create": (i32, [i32, C.POINTER(vp)]),
        "hrt_context_destroy": (i32, [vp]),
        "hrt_context_last_error": (C.c_char_p, [vp]),
        "hrt_status_string": (C.c_char_p, [i32]),
        "hrt_version": (C.c_char_p, []),
        "hrt_scene_create": (i32, [vp, C.c_char_p, C.POINTER(vp)]),
        "hrt_scene_destroy": (i32, [vp]),
        "hrt_clear_geom": (i32, [vp]),
        "hrt_add_geom_triangles3f": (i32, [vp, vp, u64, vp, u64, i32, u64, C.POINTER(u32)]),
        "hrt_update_geom_triangles3f": (i32, [vp, u32, vp, u64, vp, u64, i32, u64]),
        "hrt_clear_scene": (i32, [vp]),
        "hrt_add_instance": (i32, [vp, u32, vp, C.POINTER(u32)]),
        "hrt_update_instance": (i32, [vp, u32, vp]),
        "hrt_commit_scene": (i32, [vp, i32]),
        "hrt_query_nearest": (i32, [vp, vp, u64, vp, vp]),
        "hrt_query_any": (i32, [vp, vp, u64, vp, vp]),
        "hrt_query_nearest_host": (i32, [vp, vp, u64, vp]),
        "hrt_query_any_host": (i32, [vp, vp, u64, vp]),
        "hrt_query_nearest_host_async": (i32, [vp, vp, u64, vp, vp]),
        "hrt_query_any_host_async": (i32, [vp, vp, u64, vp, vp]),
        "hrt_scene_check": (i32, [vp]),
        "hrt_query_counters": (i32, [vp, i32, vp, u64, vp, vp]),
        "hrt_get_geom_num": (i32, [vp, C.POINTER(u32)]),
        "hrt_get_inst_num": (i32, [vp, C.POINTER(u32)]),
        "hrt_get_geom_boxes": (i32, [vp, vp, u32]),
        "hrt_geom_info": (i32, [vp, u32, vp, C.POINTER(C.c_float)]),
        "hrt_geom_export": (i32, [vp, u32, i32, vp, u64, C.POINTER(u64)]),
        "hrt_host_alloc": (i32, [u64, C.POINTER(vp)]),
        "hrt_host_free": (i32, [vp]),
        "hrt_scene_set_layout": (i32, [vp, i32]),
        "hrt_scene_set_option": (i32, [vp, i32, i32]),
        "hrt_scene_get_layout": (i32, [vp, C.POINTER(i32)]),
        "hrt_scene_set_trace_config": (i32, [vp, i32, C.POINTER(TraceConfig)]),
        "hrt_scene_get_trace_config": (i32, [vp, i32, C.POINTER(TraceConfig)]),
        "hrt_add_geoms_triangles3f_batched": (i32, [vp, u32, vp, vp, vp, vp, i32, u64, C.POINTER(u32)]),
        "hrt_query_multi": (i32, [vp, C.POINTER(QueryDesc), vp]),
        "hrt_graph_create": (i32, [vp, C.POINTER(QueryDesc), u32, C.POINTER(vp)]),
        "hrt_graph_launch": (i32, [vp, vp]),
        "hrt_graph_destroy": (i32, [vp]),
        "hrt_scene_autotune": (i32, [vp, C.POINTER(QueryDesc), i32, C.POINTER(TraceConfig), C.POINTER(C.c_float)]),
        "hrt_server_create": (i32, [vp, C.POINTER(ServerConfig), C.POINTER(vp)]),
        "hrt_server_destroy": (i32, [vp]),
        "hrt_server_add_scene": (i32, [vp, vp, u64, vp, u64, u64, i32, C.POINTER(u32)]),
        "hrt_server_scene_state": (i32, [vp, u32, C.c_double, C.POINTER(i32)]),
        "hrt_server_remove_scene": (i32, [vp, u32]),
        "hrt_server_submit": (i32, [vp, u32, i32, vp, u64, vp, C.POINTER(u64)]),
        "hrt_server_wait": (i32, [vp, u64, C.c_double, C.POINTER(RequestInfo)]),
        "hrt_server_get_stats": (i32, [vp, C.POINTER(ServerStats)]),
        "hrt_server_scene_bytes": (i32, [vp, u64, u64, C.POINTER(u64)]),
        "hrt_gen_eye_rays": (i32, [vp, vp, vp, u32, u32, C.c_float, C.c_float, vp, vp]),
        "hrt_vsgf_info": (i32, [C.c_char_p, C.POINTER(u64), C.POINTER(u64), C.POINTER(u32)]),
        "hrt_vsgf_read": (i32, [C.c_char_p, vp, vp, vp]),
        "hrt_vsgf_write": (i32, [C.c_char_p, vp, u64, vp, u64]),
        "hrt_geom_save": (i32, [vp, u32, C.c_char_p]),
        "hrt_geom_load": (i32, [vp, C.c_char_p, C.POINTER(u32)]),
        "hrt_gen_pinhole_rays": (i32, [vp, vp, vp, vp, C.c_float, u32, u32, C.c_float, C.c_float, vp, vp]),
        "hrt_gen_ao_rays": (i32, [vp, u64, vp, vp, u64, u32, C.c_float, C.c_float, vp, vp, u64, C.POINTER(u64), vp]),
        "hrt_frame_create": (i32, [vp, C.POINTER(vp)]),
        "hrt_frame_destroy": (i32, [vp]),
        "hrt_frame_render_eye": (i32, [vp, vp, vp, vp, u32, u32, vp, vp]),
        "hrt_rtao_qmc_table": (i32, [vp]),
        "hrt_rtao_qmc_tile": (i32, [u32, vp]),
        "hrt_frame_set_ao_tile": (i32, [vp, vp, u32]),
        "hrt_frame_set_normals": (i32, [vp, u32, vp, u64]),
        "hrt_frame_render_rtao": (i32, [vp, vp, C.POINTER(RtaoParams), vp, vp, vp]),
        "hrt_frame_get_buffer": (i32, [vp, i32, C.POINTER(vp), C.POINTER(u64)]),
        "hrt_frame_read_buffer": (i32, [vp, i32, vp, u64, C.POINTER(u64)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Context:
    """One GPU (hrt_context)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        st = lib().hrt_context_create(device, C.byref(self._h))
        if st != HRT_OK:
            raise HrtError(st, f"hrt_context_create({device}): {lib().hrt_status_string(st).decode()}")

    @property
    def handle(self):
        return self._h

    def last_error(self) -> str:
        return lib().hrt_context_last_error(self._h).decode()

    def check(self, st: int, what: str):
        if st != HRT_OK:
            raise HrtError(st, f"{what}: {self.last_error() or lib().hrt_status_string(st).decode()}")

    def gen_eye_rays(self, proj_inv, world_view_inv, width: int, height: int, t_near: float, t_far: float,
                     rays_ptr: int, stream: int = 0):
        """The renderers' eye rays on the device (hrt_gen_eye_rays); matrices 4x4 row-major numpy."""
        pi = np.ascontiguousarray(np.asarray(proj_inv, np.float32).T)
        wi = np.ascontiguousarray(np.asarray(world_view_inv, np.float32).T)
        self.check(lib().hrt_gen_eye_rays(self._h, _ptr(pi), _ptr(wi), width, height, t_near, t_far,
                                          C.c_void_p(rays_ptr), C.c_void_p(stream)), "hrt_gen_eye_rays")

    def gen_pinhole_rays(self, eye, target, up, fov_deg: float, width: int, height: int, tmin: float, tmax: float,
                         rays_ptr: int, stream: int = 0):
        """The benchmark camera's eye rays on the device (hrt_gen_pinhole_rays)."""
        e, t, u = (np.ascontiguousarray(x, dtype=np.float32) for x in (eye, target, up))
        self.check(lib().hrt_gen_pinhole_rays(self._h, _ptr(e), _ptr(t), _ptr(u), fov_deg, width, height, tmin, tmax,
                                              C.c_void_p(rays_ptr), C.c_void_p(stream)), "hrt_gen_pinhole_rays")

    def close(self):
        if self._h:
            lib().hrt_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _as_rays(posAndNear, dirAndFar=None) -> np.ndarray:
    """Interleaved float32 [n, 8] rays from (pos, dir) float4 arrays or an [n, 8] array."""
    if dirAndFar is None:
        r = np.ascontiguousarray(posAndNear, dtype=np.float32).reshape(-1, 8)
        return r
    p = np.asarray(posAndNear, dtype=np.float32).reshape(-1, 4)
    d = np.asarray(dirAndFar, dtype=np.float32).reshape(-1, 4)
    if p.shape != d.shape:
        raise ValueError("posAndNear and dirAndFar must have the same length")
    return np.ascontiguousarray(np.concatenate([p, d], axis=1))


class SceneRT:
    """GPU LBVH scene behind HeavyRT's ISceneObject interface (core/CrossRT.h:64-193)."""

    def __init__(self, ctx: Context | None = None, build_name: str = "cbvh_lbvh", layout=LAYOUT_BVH2,
                 triangle_test=TRI_MOLLER_TRUMBORE):
        self.ctx = ctx or default_context()
        self._h = C.c_void_p()
        self.ctx.check(lib().hrt_scene_create(self.ctx.handle, build_name.encode() if build_name else None,
                                              C.byref(self._h)), "hrt_scene_create")
        self._build_name = build_name
        if isinstance(layout, str):
            if layout.lower() not in LAYOUT_NAMES:
                raise HrtError(HRT_ERR_UNSUPPORTED, f"layout '{layout}' is not provided by this engine")
            layout = LAYOUT_NAMES[layout.lower()]
        if layout != LAYOUT_BVH2:
            self.ctx.check(lib().hrt_scene_set_layout(self._h, int(layout)), "set_layout")
        if isinstance(triangle_test, str):
            triangle_test = TRI_TEST_NAMES[triangle_test.lower()]
        if triangle_test != TRI_MOLLER_TRUMBORE:
            self.set_triangle_test(triangle_test)

    def set_bvh4_merge(self, value: int):
        """0: the reference's leaf merge rule; M: merge subtrees of <= M triangles."""
        self.ctx.check(lib().hrt_scene_set_option(self._h, OPTION_BVH4_MERGE, int(value)), "set_option")

    def set_tlas(self, enabled: bool):
        """Instance tree over the instances (default on; takes effect at CommitScene)."""
        self.ctx.check(lib().hrt_scene_set_option(self._h, OPTION_TLAS, int(bool(enabled))), "set_option")

    def set_l2_persist(self, mib: int):
        """Keep the node array in L2 for queries (persisting set-aside of `mib` MiB; 0 off)."""
        self.ctx.check(lib().hrt_scene_set_option(self._h, OPTION_L2_PERSIST, int(mib)), "set_option")

    def set_morton_frame(self, frame: int):
        """MORTON_PER_AXIS (the reference's grid) or MORTON_CUBIC, for geometry added afterwards."""
        self.ctx.check(lib().hrt_scene_set_option(self._h, OPTION_MORTON_FRAME, int(frame)), "set_option")

    def set_bvh4_collapse(self, rule: int):
        """BVH4_COLLAPSE_EVEN_DEPTH (the reference's BVH2ToBVH4 rule) or
        BVH4_COLLAPSE_LARGEST_FIRST, for geometry added afterwards."""
        self.ctx.check(lib().hrt_scene_set_option(self._h, OPTION_BVH4_COLLAPSE, int(rule)), "set_option")

    def set_triangle_test(self, test: int):
        """TRI_MOLLER_TRUMBORE (the reference's test) or TRI_WATERTIGHT; before the first geometry."""
        self.ctx.check(lib().hrt_scene_set_option(self._h, OPTION_TRIANGLE_TEST, int(test)), "set_option")

    @property
    def layout(self) -> int:
        v = C.c_int()
        self.ctx.check(lib().hrt_scene_get_layout(self._h, C.byref(v)), "get_layout")
        return v.value

    # ---- ISceneObject ---------------------------------------------------
    def Name(self) -> str:  # ISceneObject::Name, core/CrossRT.h:72
        return "GB300_LBVH"

    def BuildName(self) -> str:  # core/CrossRT.h:77
        return self._build_name

    def ClearGeom(self):  # core/CrossRT.h:82
        self.ctx.check(lib().hrt_clear_geom(self._h), "ClearGeom")

    def AddGeom_Triangles3f(self, a_vpos3f, a_vertNumber=None, a_triIndices=None, a_indNumber=None,
                            a_qualityLevel=BUILD_HIGH, vByteStride=12) -> int:  # core/CrossRT.h:94
        v = np.ascontiguousarray(a_vpos3f, dtype=np.float32)
        idx = np.ascontiguousarray(a_triIndices, dtype=np.uint32).reshape(-1)
        stride = int(vByteStride) if vByteStride else 12
        if a_vertNumber is None:
            a_vertNumber = v.size * 4 // stride
        if a_indNumber is None:
            a_indNumber = idx.size
        if v.size * 4 < a_vertNumber * stride - (stride - 12):
            raise ValueError("vertex array smaller than a_vertNumber * vByteStride")
        gid = C.c_uint32()
        self.ctx.check(lib().hrt_add_geom_triangles3f(self._h, _ptr(v), int(a_vertNumber), _ptr(idx), int(a_indNumber),
                                                      int(a_qualityLevel), stride, C.byref(gid)),
                       "AddGeom_Triangles3f")
        return gid.value

    def UpdateGeom_Triangles3f(self, a_geomId, a_vpos3f, a_vertNumber, a_triIndices, a_indNumber,
                               a_qualityLevel=BUILD_HIGH, vByteStride=12):  # core/CrossRT.h:105
        v = np.ascontiguousarray(a_vpos3f, dtype=np.float32)
        idx = np.ascontiguousarray(a_triIndices, dtype=np.uint32)
        self.ctx.check(lib().hrt_update_geom_triangles3f(self._h, a_geomId, _ptr(v), a_vertNumber, _ptr(idx), a_indNumber,
                                                         a_qualityLevel, vByteStride), "UpdateGeom_Triangles3f")

    def ClearScene(self):  # core/CrossRT.h:110
        self.ctx.check(lib().hrt_clear_scene(self._h), "ClearScene")

    def CommitScene(self, a_qualityLevel=BUILD_MEDIUM):  # core/CrossRT.h:115
        self.ctx.check(lib().hrt_commit_scene(self._h, int(a_qualityLevel)), "CommitScene")

    def AddInstance(self, a_geomId: int, a_matrix=None) -> int:  # core/CrossRT.h:123
        m = np.eye(4, dtype=np.float32) if a_matrix is None else np.asarray(a_matrix, dtype=np.float32).reshape(4, 4)
        col = np.ascontiguousarray(m.T)  # column-major storage
        iid = C.c_uint32()
        self.ctx.check(lib().hrt_add_instance(self._h, a_geomId, _ptr(col), C.byref(iid)), "AddInstance")
        return iid.value

    def UpdateInstance(self, a_instanceId: int, a_matrix):  # core/CrossRT.h:130
        col = np.ascontiguousarray(np.asarray(a_matrix, dtype=np.float32).reshape(4, 4).T)
        self.ctx.check(lib().hrt_update_instance(self._h, a_instanceId, _ptr(col)), "UpdateInstance")

    def RayQuery_NearestHit(self, posAndNear, dirAndFar=None) -> np.ndarray:  # core/CrossRT.h:143 (batched)
        rays = _as_rays(posAndNear, dirAndFar)
        out = np.empty(rays.shape[0], dtype=HIT_DTYPE)
        self.ctx.check(lib().hrt_query_nearest_host(self._h, _ptr(rays), rays.shape[0], _ptr(out)), "RayQuery_NearestHit")
        return out

    def RayQuery_AnyHit(self, posAndNear, dirAndFar=None) -> np.ndarray:  # core/CrossRT.h:151 (batched)
        rays = _as_rays(posAndNear, dirAndFar)
        out = np.empty(rays.shape[0], dtype=np.uint8)
        self.ctx.check(lib().hrt_query_any_host(self._h, _ptr(rays), rays.shape[0], _ptr(out)), "RayQuery_AnyHit")
        return out.astype(bool)

    def GetGeomNum(self) -> int:  # core/CrossRT.h:163
        n = C.c_uint32()
        self.ctx.check(lib().hrt_get_geom_num(self._h, C.byref(n)), "GetGeomNum")
        return n.value

    def GetInstNum(self) -> int:  # core/CrossRT.h:164
        n = C.c_uint32()
        self.ctx.check(lib().hrt_get_inst_num(self._h, C.byref(n)), "GetInstNum")
        return n.value

    def GetGeomBoxes(self) -> np.ndarray:  # core/CrossRT.h:165, float4 pairs (boxMin, boxMax)
        n = self.GetGeomNum()
        out = np.empty((n, 8), dtype=np.float32)
        self.ctx.check(lib().hrt_get_geom_boxes(self._h, _ptr(out), n), "GetGeomBoxes")
        return out

    # ---- engine extensions ----------------------------------------------
    def add_geoms_batched(self, verts_list, idx_list, a_qualityLevel=BUILD_HIGH) -> list:
        """Builds many geometries with one segmented build; returns their ids.

        verts_list[i]: float32 [V_i, 3] or [V_i, 4] (xyz used); idx_list[i]: uint32 indices local to
        verts_list[i]."""
        if len(verts_list) != len(idx_list) or not verts_list:
            raise ValueError("verts_list and idx_list must be non-empty and of equal length")
        vs = []
        for v in verts_list:
            a = np.asarray(v, dtype=np.float32)
            a = a.reshape(len(a), -1) if a.size else np.zeros((0, 4), np.float32)
            if a.shape[1] != 4:  # the engine reads xyz at a 16-byte stride; w is not used
                p4 = np.ones((len(a), 4), np.float32)
                p4[:, :3] = a[:, :3]
                a = p4
            vs.append(a)
        v = np.concatenate(vs, axis=0) if len(vs) > 1 else np.ascontiguousarray(vs[0])
        ids = [np.asarray(i, dtype=np.uint32).reshape(-1) for i in idx_list]
        idx = np.ascontiguousarray(np.concatenate(ids))
        voff = np.zeros(len(vs) + 1, dtype=np.uint64)
        voff[1:] = np.cumsum([len(x) for x in vs])
        ioff = np.zeros(len(ids) + 1, dtype=np.uint64)
        ioff[1:] = np.cumsum([len(x) for x in ids])
        first = C.c_uint32()
        self.ctx.check(lib().hrt_add_geoms_triangles3f_batched(self._h, len(vs), _ptr(v), _ptr(voff), _ptr(idx),
                                                               _ptr(ioff), int(a_qualityLevel), 16, C.byref(first)),
                       "add_geoms_batched")
        return list(range(first.value, first.value + len(vs)))

    def gen_ao_rays(self, seed: int, eye_ptr: int, hits_ptr: int, n_eye: int, per_hit: int, length: float,
                    offset: float, out_ptr: int, capacity: int, owner_ptr: int = 0, stream: int = 0) -> int:
        """AO rays from device eye rays and their hits (hrt_gen_ao_rays); returns the count."""
        n = C.c_uint64()
        self.ctx.check(lib().hrt_gen_ao_rays(self._h, seed, C.c_void_p(eye_ptr), C.c_void_p(hits_ptr), n_eye, per_hit,
                                             length, offset, C.c_void_p(out_ptr), C.c_void_p(owner_ptr or None),
                                             capacity, C.byref(n), C.c_void_p(stream)), "hrt_gen_ao_rays")
        return n.value

    def save_geom(self, geom_id: int, path) -> None:
        """Writes a BVH blob of a built geometry (hrt_geom_save)."""
        self.ctx.check(lib().hrt_geom_save(self._h, geom_id, str(path).encode()), "hrt_geom_save")

    def load_geom(self, path) -> int:
        """Restores a geometry from a BVH blob without building (hrt_geom_load); returns its id."""
        gid = C.c_uint32()
        self.ctx.check(lib().hrt_geom_load(self._h, str(path).encode(), C.byref(gid)), "hrt_geom_load")
        return gid.value

    def query_multi(self, desc: QueryDesc, stream: int = 0):
        """Asynchronous (optionally segmented) query on device arrays (hrt_query_multi)."""
        self.ctx.check(lib().hrt_query_multi(self._h, C.byref(desc), C.c_void_p(stream)), "query_multi")

    def autotune(self, desc: QueryDesc, repeats: int = 3):
        """Sweeps the launch grid for desc's kind, keeps the fastest; returns (config dict, ms)."""
        best = TraceConfig()
        ms = C.c_float()
        self.ctx.check(lib().hrt_scene_autotune(self._h, C.byref(desc), int(repeats), C.byref(best), C.byref(ms)),
                       "autotune")
        return best.as_dict(), ms.value

    def capture(self, descs) -> "QueryGraph":
        """Records the launches of `descs` (QueryDesc list) into a CUDA graph (hrt_graph_create)."""
        return QueryGraph(self, descs)


    def query_device(self, kind: int, rays_ptr: int, n: int, out_ptr: int, stream: int = 0):
        """Asynchronous query on device arrays (kind 0 nearest -> CRT_Hit[n], 1 any -> uint8[n])."""
        f = lib().hrt_query_nearest if kind == 0 else lib().hrt_query_any
        self.ctx.check(f(self._h, C.c_void_p(rays_ptr), n, C.c_void_p(out_ptr), C.c_void_p(stream)), "query")

    def query_counters(self, kind: int, rays_ptr: int, n: int, stream: int = 0):
        c = (C.c_uint64 * 2)()
        self.ctx.check(lib().hrt_query_counters(self._h, kind, C.c_void_p(rays_ptr), n, c, C.c_void_p(stream)),
                       "query_counters")
        return int(c[0]), int(c[1])

    def set_trace_config(self, kind: int, threadsPerBlock=128, persistent=1, stepsPerRefill=16, refillLanes=24,
                         stackEntries=0, imageWidth=0):
        c = TraceConfig(threadsPerBlock, persistent, stepsPerRefill, refillLanes, stackEntries, imageWidth)
        self.ctx.check(lib().hrt_scene_set_trace_config(self._h, kind, C.byref(c)), "set_trace_config")

    def trace_config(self, kind: int) -> dict:
        c = TraceConfig()
        self.ctx.check(lib().hrt_scene_get_trace_config(self._h, kind, C.byref(c)), "trace_config")
        return c.as_dict()

    def geom_info(self, geom_id: int = 0) -> dict:
        out = (C.c_uint64 * 4)()
        ms = C.c_float()
        self.ctx.check(lib().hrt_geom_info(self._h, geom_id, out, C.byref(ms)), "geom_info")
        return {"tris": out[0], "leaves": out[1], "pairs": out[2], "bytes": out[3], "build_ms": ms.value}

    def export(self, geom_id: int, what: int) -> np.ndarray:
        size = C.c_uint64()
        self.ctx.check(lib().hrt_geom_export(self._h, geom_id, what, None, 0, C.byref(size)), "export size")
        dt = np.dtype(_EXPORT_DTYPES[what])
        out = np.empty(size.value // dt.itemsize, dtype=dt)
        if size.value:
            self.ctx.check(lib().hrt_geom_export(self._h, geom_id, what, _ptr(out), size.value, C.byref(size)), "export")
        return out

    def close(self):
        if self._h:
            lib().hrt_scene_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class QueryGraph:
    """A captured sequence of queries (hrt_graph); launch() replays it on a stream."""

    def __init__(self, scene: SceneRT, descs):
        self.scene = scene
        arr = (QueryDesc * len(descs))(*descs)
        self._descs = arr
        self._h = C.c_void_p()
        scene.ctx.check(lib().hrt_graph_create(scene._h, arr, len(descs), C.byref(self._h)), "hrt_graph_create")

    def launch(self, stream: int = 0):
        self.scene.ctx.check(lib().hrt_graph_launch(self._h, C.c_void_p(stream)), "hrt_graph_launch")

    def close(self):
        if self._h:
            lib().hrt_graph_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop over resident scenes (hrt_server_*): builds on arrival,
    memory-budget admission, continuous batching of ray requests."""

    def __init__(self, ctx: Context | None = None, memory_budget: int = 0, slot_rays: int = 0, slots: int = 0,
                 max_scenes: int = 0, max_batch_requests: int = 0, layout=LAYOUT_BVH2, bvh4_merge: int = 0,
                 morton_frame: int = MORTON_PER_AXIS, bvh4_collapse: int = BVH4_COLLAPSE_EVEN_DEPTH):
        self.ctx = ctx or default_context()
        if isinstance(layout, str):
            layout = LAYOUT_NAMES[layout.lower()]
        cfg = ServerConfig(memory_budget, slot_rays, slots, max_scenes, max_batch_requests, int(layout),
                           int(bvh4_merge), int(morton_frame), int(bvh4_collapse))
        self._h = C.c_void_p()
        self.ctx.check(lib().hrt_server_create(self.ctx.handle, C.byref(cfg), C.byref(self._h)), "hrt_server_create")

    def add_scene(self, verts: np.ndarray, idx: np.ndarray, evictable: bool = True) -> int:
        """Queues a scene build; returns its id at once.  verts: float32 [V, 3] or [V, 4]."""
        v = np.ascontiguousarray(verts, dtype=np.float32)
        v = v.reshape(v.shape[0], -1) if v.size else v.reshape(0, 3)
        i = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1)
        sid = C.c_uint32()
        self.ctx.check(lib().hrt_server_add_scene(self._h, _ptr(v), v.shape[0], _ptr(i), i.size, 4 * v.shape[1],
                                                  int(bool(evictable)), C.byref(sid)), "hrt_server_add_scene")
        return sid.value

    def scene_state(self, scene_id: int, timeout: float = 0.0) -> int:
        st = C.c_int()
        self.ctx.check(lib().hrt_server_scene_state(self._h, scene_id, float(timeout), C.byref(st)), "scene_state")
        return st.value

    def remove_scene(self, scene_id: int):
        self.ctx.check(lib().hrt_server_remove_scene(self._h, scene_id), "hrt_server_remove_scene")

    def submit(self, scene_id: int, kind: int, rays_ptr: int, n: int, out_ptr: int) -> int:
        """Queues a request on host buffers (pointers as ints); returns its ticket."""
        t = C.c_uint64()
        self.ctx.check(lib().hrt_server_submit(self._h, scene_id, kind, C.c_void_p(rays_ptr), n, C.c_void_p(out_ptr),
                                               C.byref(t)), "hrt_server_submit")
        return t.value

    def submit_array(self, scene_id: int, kind: int, rays: np.ndarray, out: np.ndarray) -> int:
        return self.submit(scene_id, kind, rays.ctypes.data, rays.shape[0], out.ctypes.data)

    def wait(self, ticket: int, timeout: float = -1.0):
        """(status, info dict) of a request; status HRT_ERR_TIMEOUT keeps the ticket valid."""
        info = RequestInfo()
        st = lib().hrt_server_wait(self._h, ticket, float(timeout), C.byref(info))
        return st, info.as_dict()

    def stats(self) -> dict:
        s = ServerStats()
        self.ctx.check(lib().hrt_server_get_stats(self._h, C.byref(s)), "hrt_server_get_stats")
        return s.as_dict()

    def scene_bytes(self, n_verts: int, n_tris: int) -> int:
        b = C.c_uint64()
        self.ctx.check(lib().hrt_server_scene_bytes(self._h, n_verts, n_tris, C.byref(b)), "hrt_server_scene_bytes")
        return b.value

    def close(self):
        if self._h:
            lib().hrt_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


AO_TILE_SIZE = 128
HRT_MAX_AO_RAYS_PER_PIXEL = 1024
FRAME_EYE_RAYS, FRAME_RAY_PIXEL, FRAME_EYE_HITS, FRAME_POSITIONS = 0, 1, 2, 3
FRAME_VISIBILITY, FRAME_AO_PIXEL, FRAME_AO_RAYS, FRAME_AO_HITS = 4, 5, 6, 7


def rtao_qmc_table() -> np.ndarray:
    """The direction numbers of RTAO's quasi-random generator (hrt_rtao_qmc_table), uint32 [4, 31]."""
    out = np.empty((4, 31), np.uint32)
    st = lib().hrt_rtao_qmc_table(_ptr(out))
    if st != HRT_OK:
        raise HrtError(st, "hrt_rtao_qmc_table")
    return out


def rtao_qmc_tile(rays_per_pixel: int) -> np.ndarray:
    """RTAO's 128x128 AO sample tile (hrt_rtao_qmc_tile): float32 [128*128*R, 2]."""
    out = np.empty((AO_TILE_SIZE * AO_TILE_SIZE * rays_per_pixel, 2), np.float32)
    st = lib().hrt_rtao_qmc_tile(rays_per_pixel, _ptr(out))
    if st != HRT_OK:
        raise HrtError(st, f"hrt_rtao_qmc_tile({rays_per_pixel})")
    return out


class Frame:
    """Frames of HeavyRT's example renderers on the device (hrt_frame): colours go to
    a device buffer (a pointer), the frame's own buffers stay on the device."""

    _BUF = {FRAME_EYE_RAYS: (np.float32, 8), FRAME_RAY_PIXEL: (np.uint32, 1), FRAME_EYE_HITS: (np.uint32, 8),
            FRAME_POSITIONS: (np.float32, 4), FRAME_VISIBILITY: (np.float32, 1), FRAME_AO_PIXEL: (np.uint32, 1),
            FRAME_AO_RAYS: (np.float32, 8), FRAME_AO_HITS: (np.uint8, 1)}

    def __init__(self, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self._h = C.c_void_p()
        self.ctx.check(lib().hrt_frame_create(self.ctx.handle, C.byref(self._h)), "hrt_frame_create")

    def render_eye(self, scene: "SceneRT", proj_inv, world_view_inv, width: int, height: int, colors_ptr: int,
                   stream: int = 0):
        pi = np.ascontiguousarray(np.asarray(proj_inv, np.float32).T)
        wi = np.ascontiguousarray(np.asarray(world_view_inv, np.float32).T)
        self.ctx.check(lib().hrt_frame_render_eye(self._h, scene._h, _ptr(pi), _ptr(wi), width, height,
                                                  C.c_void_p(colors_ptr), C.c_void_p(stream)), "hrt_frame_render_eye")

    def set_ao_tile(self, tile: np.ndarray, rays_per_pixel: int):
        t = np.ascontiguousarray(tile, np.float32)
        if t.size != AO_TILE_SIZE * AO_TILE_SIZE * rays_per_pixel * 2:
            raise ValueError("tile must hold 128*128*rays_per_pixel float pairs")
        self.ctx.check(lib().hrt_frame_set_ao_tile(self._h, _ptr(t), rays_per_pixel), "hrt_frame_set_ao_tile")

    def set_normals(self, geom_id: int, normals: np.ndarray):
        nn = np.ascontiguousarray(normals, np.float32).reshape(-1, 4)
        self.ctx.check(lib().hrt_frame_set_normals(self._h, geom_id, _ptr(nn), nn.shape[0]), "hrt_frame_set_normals")

    def render_rtao(self, scene: "SceneRT", proj_inv, world_view_inv, width: int, height: int, colors_ptr: int,
                    z_near: float = 0.0, z_far: float = 3.4028234663852886e38, ao_max_radius: float = 2.0,
                    power: float = 1.0, norm_matrices=None, stream: int = 0):
        """norm_matrices: (nInst, 4, 4) row-major (identity for every instance when None)."""
        p = RtaoParams()
        p.projInv[:] = np.asarray(proj_inv, np.float32).T.reshape(-1).tolist()
        p.worldViewInv[:] = np.asarray(world_view_inv, np.float32).T.reshape(-1).tolist()
        p.zNear, p.zFar, p.width, p.height = z_near, z_far, width, height
        p.aoMaxRadius, p.power = ao_max_radius, power
        n_inst = scene.GetInstNum()
        if norm_matrices is None:
            norm_matrices = np.broadcast_to(np.eye(4, dtype=np.float32), (max(n_inst, 1), 4, 4))
        nm = np.ascontiguousarray(np.transpose(np.asarray(norm_matrices, np.float32).reshape(-1, 4, 4), (0, 2, 1)))
        self.ctx.check(lib().hrt_frame_render_rtao(self._h, scene._h, C.byref(p), _ptr(nm), C.c_void_p(colors_ptr),
                                                   C.c_void_p(stream)), "hrt_frame_render_rtao")

    def buffer(self, which: int):
        """(device pointer, count, numpy dtype, values per entry) of one of the last frame's buffers."""
        d, n = C.c_void_p(), C.c_uint64()
        self.ctx.check(lib().hrt_frame_get_buffer(self._h, which, C.byref(d), C.byref(n)), "hrt_frame_get_buffer")
        dt, per = self._BUF[which]
        return (d.value or 0), int(n.value), dt, per

    def read(self, which: int) -> np.ndarray:
        """A copy of one of the last frame's buffers on the host: (count, values) or (count,)."""
        _, n, dt, per = self.buffer(which)
        out = np.empty((n, per) if per > 1 else n, dt)
        nb = C.c_uint64()
        self.ctx.check(lib().hrt_frame_read_buffer(self._h, which, _ptr(out), out.nbytes, C.byref(nb)),
                       "hrt_frame_read_buffer")
        return out

    def close(self):
        if self._h:
            lib().hrt_frame_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_vsgf(path, normals: bool = False):
    """A VSGF mesh (hrt_vsgf_read): float32 [V, 4] positions (w = 1), uint32 indices
    (and float32 [V, 4] normals when asked)."""
    nv, ni, fl = C.c_uint64(), C.c_uint64(), C.c_uint32()
    st = lib().hrt_vsgf_info(str(path).encode(), C.byref(nv), C.byref(ni), C.byref(fl))
    if st != HRT_OK:
        raise HrtError(st, f"hrt_vsgf_info({path}): not a readable VSGF mesh")
    v = np.empty((nv.value, 4), np.float32)
    idx = np.empty(ni.value, np.uint32)
    nrm = np.empty((nv.value, 4), np.float32) if normals else None
    st = lib().hrt_vsgf_read(str(path).encode(), _ptr(v), _ptr(idx), _ptr(nrm) if normals else None)
    if st != HRT_OK:
        raise HrtError(st, f"hrt_vsgf_read({path})")
    return (v, idx, nrm) if normals else (v, idx)


def save_vsgf(path, verts, idx):
    """Writes positions + indices as a VSGF mesh (hrt_vsgf_write)."""
    v = np.ascontiguousarray(np.asarray(verts, np.float32).reshape(-1, np.asarray(verts).shape[-1]))
    if v.shape[1] == 3:
        v = np.ascontiguousarray(np.concatenate([v, np.ones((len(v), 1), np.float32)], axis=1))
    i = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1)
    st = lib().hrt_vsgf_write(str(path).encode(), _ptr(v), len(v), _ptr(i), i.size)
    if st != HRT_OK:
        raise HrtError(st, f"hrt_vsgf_write({path})")


def CreateSceneRT(a_implName: str = "GB300_LBVH", a_buildName: str = "cbvh_lbvh", a_layoutName: str = "") -> SceneRT:
    """Factory mirroring CreateSceneRT (core/FactoryRT.cpp:29-78, core/CrossRT.h:195)."""
    if a_implName not in ("GB300_LBVH", "BVH2Common"):
        raise HrtError(HRT_ERR_UNSUPPORTED, f"implementation '{a_implName}' is not provided by this engine")
    return SceneRT(build_name=a_buildName, layout=a_layoutName or "")


def DeleteSceneRT(scene: SceneRT):  # core/CrossRT.h:196
    scene.close()


class PinnedBuffer:
    """Page-locked host buffer (hrt_host_alloc) viewed as a numpy array."""

    def __init__(self, nbytes: int):
        self._p = C.c_void_p()
        st = lib().hrt_host_alloc(nbytes, C.byref(self._p))
        if st != HRT_OK:
            raise HrtError(st, "hrt_host_alloc")
        self.nbytes = nbytes

    def array(self, dtype, count=None) -> np.ndarray:
        dt = np.dtype(dtype)
        count = self.nbytes // dt.itemsize if count is None else count
        buf = (C.c_char * (count * dt.itemsize)).from_address(self._p.value)
        return np.frombuffer(buf, dtype=dt, count=count)

    @property
    def ptr(self) -> int:
        return self._p.value

    def free(self):
        if self._p:
            lib().hrt_host_free(self._p)
            self._p = C.c_void_p()
